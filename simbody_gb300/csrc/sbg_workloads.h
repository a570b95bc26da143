/* sbg_workloads.h -- seeded synthetic workloads (host only) shaped like the
 * benchmark configurations of the batched forward-dynamics path. Used by the
 * tests, bench.py and the C++ examples to build identical inputs for the GPU
 * engine and the CPU oracle. Pointers stay valid until sbg_workload_destroy. */
#ifndef SBG_WORKLOADS_H_
#define SBG_WORKLOADS_H_
#include <stdint.h>
#include "../../include/simbody_gb300.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct sbg_workload_s* sbg_workload;
const char* sbg_workload_last_error(void);
int sbg_workload_create(int32_t config, int32_t ninstances, sbg_workload* out);
int sbg_workload_destroy(sbg_workload w);
int32_t sbg_workload_num_systems(sbg_workload w);
int32_t sbg_workload_num_instances(sbg_workload w);
const sbg_system_desc* sbg_workload_systems(sbg_workload w);
const int32_t* sbg_workload_instance_system(sbg_workload w);
const int64_t* sbg_workload_y_offsets(sbg_workload w);   /* ninstances + 1 */
const double* sbg_workload_y0(sbg_workload w);
double sbg_workload_h(sbg_workload w);
int32_t sbg_workload_nsteps(sbg_workload w);
const int32_t* sbg_workload_horizons(sbg_workload w);    /* serving only */
const double* sbg_workload_arrivals(sbg_workload w);     /* serving only */
#ifdef __cplusplus
}
#endif
#endif
