/* sbg_oracle_api.h -- C API of the CPU oracle (test infrastructure only). */
#ifndef SBG_ORACLE_API_H_
#define SBG_ORACLE_API_H_
#include <stdint.h>
#include "../include/simbody_gb300.h"
#ifdef __cplusplus
extern "C" {
#endif
const char* oracle_last_error(void);
int oracle_system_sizes(const sbg_system_desc* d, int32_t* nq, int32_t* nu, int32_t* nquat);
int oracle_realize_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                         const int64_t* y_off, const double* y, double* ydot, int32_t* status, int32_t nthreads);
int oracle_minv_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                      const int64_t* y_off, const double* y, const int64_t* u_off, const double* f, double* out,
                      int32_t nthreads);
int oracle_rk_merson_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                           const int64_t* y_off, double* y, double* t, double h, int32_t nsteps, double accuracy,
                           double consTol, int32_t projectEveryStep, int32_t* status, int64_t* nproj,
                           int32_t nthreads);
int oracle_rk_merson_run_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                               const int64_t* y_off, double* y, double* t, double h, int32_t nsteps, double t_report,
                               int32_t initialize, double accuracy, double consTol, int32_t projectEveryStep,
                               int32_t* status, int32_t nthreads);
int oracle_qdotdot_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                         const int64_t* y_off, const double* y, const double* ydot, const int64_t* q_off,
                         double* qdotdot);
int oracle_tree_op_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                         const int64_t* y_off, const double* y, const int64_t* u_off, const int64_t* b_off,
                         int32_t op, const double* x, const double* fmob, const double* Fbody, double* out,
                         int32_t nthreads);
int oracle_system_forces_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                               const int64_t* y_off, const double* y, const int64_t* u_off, const int64_t* b_off,
                               double* fmob, double* Fbody, int32_t nthreads);
int oracle_rk_merson_adaptive_batch(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of,
                                    int32_t ninst, const int64_t* y_off, double* y, double* t, double tFinal,
                                    double hInit, double hMin, double hMax, double accuracy, double consTol,
                                    int32_t projectEveryStep, int32_t maxSteps, int32_t* status, int64_t* stats,
                                    int32_t nthreads);
int oracle_instance_invariants(const sbg_system_desc* d, const double* y, double* energy, double* perr, double* verr,
                               double* aerr);
int oracle_qtz_solve(int32_t nr, int32_t nc, const double* A, double rcond, const double* b, double* x);
int oracle_adjust_step_size(double err, int32_t errOrder, int32_t limited, double accuracy, double hMin, double hMax,
                            double* h);
int oracle_count_realize(const sbg_system_desc* d, const double* y, int64_t* counts);
double oracle_time_realize(const sbg_system_desc* systems, int32_t nsys, const int32_t* sys_of, int32_t ninst,
                           const int64_t* y_off, const double* y, double* ydot, int32_t nreps, int32_t nthreads);
int oracle_hardware_threads(void);
#ifdef __cplusplus
}
#endif
#endif
