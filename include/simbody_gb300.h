/* simbody_gb300.h -- C ABI of the GB300 batched forward-dynamics engine.
 *
 * This is the drop-in boundary for Simbody's O(n) articulated-body hot path:
 * a batch of states of systems built from SimbodyMatterSubsystem,
 * MobilizedBody::{Pin, Slider, Universal, Ball, Free}, Force::Gravity,
 * Force::MobilityLinearSpring / MobilityLinearDamper (and Constraint::Ball loop
 * closures) is realized through Stage::Acceleration and stepped with a
 * fixed-step Runge-Kutta-Merson integrator, on one GPU.
 *
 * Simbody itself exposes this path only through its C++ class API; each entry
 * point below names the reference call it replaces (paths are relative to the
 * Simbody source tree).
 *
 * Conventions
 *   - Every function returns an int status: 0 (SBG_OK) on success, an
 *     sbg_status code otherwise; sbg_last_error() then holds a message for the
 *     calling thread. No C++ exception crosses this boundary.
 *   - The caller owns every host buffer; the library owns all device memory.
 *   - One CUDA stream per batch. Calls on one batch handle are not re-entrant;
 *     different handles may be used from different threads.
 *   - Host state layout is Simbody's State::getY() = [q, u] per instance,
 *     instances packed back to back in batch order (sbg_batch_layout gives
 *     the offsets). Derivatives use the same packing: [qdot, udot].
 */
#ifndef SIMBODY_GB300_H_
#define SIMBODY_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SBG_ABI_VERSION 2

typedef enum sbg_status {
    SBG_OK = 0,
    SBG_ERR_INVALID = 1,      /* bad argument or ill-formed system */
    SBG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    SBG_ERR_NOMEM = 3,        /* device allocation failed */
    SBG_ERR_BUDGET = 4,       /* request exceeds the configured device budget */
    SBG_ERR_STATE = 5,        /* call out of order (e.g. no state set yet) */
    SBG_ERR_UNSUPPORTED = 6,  /* feature outside the supported subset */
    SBG_ERR_NO_DEVICE = 7     /* no CUDA device / driver */
} sbg_status;

/* Mobilizer kinds. Coordinates follow Simbody's defaults:
 *   PIN         nq=1 nu=1  rotation about Fz            (RigidBodyNodeSpec_Pin.h:103-131)
 *   SLIDER      nq=1 nu=1  translation along Fx         (RigidBodyNodeSpec_Slider.h:100-119)
 *   UNIVERSAL   nq=2 nu=2  body-fixed X then Y          (RigidBodyNodeSpec_Universal.h:124-189)
 *   BALL        nq=4 nu=3  quaternion, w_FM in F        (RigidBodyNodeSpec_Ball.h:113-214)
 *   FREE        nq=7 nu=6  [quat, p_FM], [w_FM, v_FM]   (RigidBodyNodeSpec_Free.h:142-219)
 *   GIMBAL      nq=3 nu=3  body-fixed X-Y-Z angles, u = qdot (RigidBodyNodeSpec_Gimbal.h)
 *   TRANSLATION nq=3 nu=3  p_FM = q, u = qdot           (RigidBodyNodeSpec_Translation.h)
 *   CYLINDER    nq=2 nu=2  rotation about and translation along Fz, u = qdot
 *                                                        (RigidBodyNodeSpec_Cylinder.h)
 *   PLANAR      nq=3 nu=3  rotation about Fz, translation along Fx, Fy, u = qdot
 *                                                        (RigidBodyNodeSpec_Planar.h)
 *   BUSHING     nq=6 nu=6  body-fixed X-Y-Z angles then p_FM, u = qdot
 *                                                        (RigidBodyNodeSpec_Bushing.h)
 * With SBG_SYSTEM_EULER_ANGLES a system's BALL and FREE bodies use
 * body-fixed X-Y-Z angles instead of quaternions (nq = 3 and 6; u is still
 * w_FM (, v_FM) in F): SimbodyMatterSubsystem::setUseEulerAngles
 * (RigidBodyNodeSpec_Ball.h:118-127, 198-209). */
typedef enum sbg_mobilizer {
    SBG_PIN = 0,
    SBG_SLIDER = 1,
    SBG_UNIVERSAL = 2,
    SBG_BALL = 3,
    SBG_FREE = 4,
    SBG_GIMBAL = 5,
    SBG_TRANSLATION = 6,
    SBG_CYLINDER = 7,
    SBG_PLANAR = 8,
    SBG_BUSHING = 9,
    SBG_WELD = 10,              /* no mobilities: X_FM = identity (RigidBodyNode_Weld.cpp:369-470) */
    SBG_SCREW = 11              /* 1: rotation q about Fz with translation pitch*q along it
                                   (RigidBodyNodeSpec_Screw.h:121-140) */
} sbg_mobilizer;
#define SBG_NUM_MOBILIZERS 12

/* sbg_system_desc.flags */
#define SBG_SYSTEM_EULER_ANGLES 1  /* SimbodyMatterSubsystem::setUseEulerAngles(true) */

typedef enum sbg_precision {
    SBG_PRECISION_FP64 = 0,   /* every recursion in FP64 */
    SBG_PRECISION_MIXED = 1,  /* FP32 spatial recursions + one refinement step
                                 with a double-float inverse-dynamics residual;
                                 FP64 state accumulation, quaternion
                                 normalisation and loop-closure solve */
    SBG_PRECISION_MIXED_FAST = 2  /* FP32 spatial recursions without refinement */
} sbg_precision;

/* Per-instance status bits written by the kernels (never a device trap). */
#define SBG_INST_OK                 0
#define SBG_INST_NONFINITE          1   /* NaN/Inf in a derivative or state */
#define SBG_INST_SINGULAR_D         2   /* zero pivot in a D = H^T P H inverse */
#define SBG_INST_PROJECTION_FAILED  4   /* quaternion/constraint projection refused */
#define SBG_INST_CHOLESKY_FAIL      8   /* loop-closure Gram not finite, or all zero (closures no
                                               mobility can move); redundant closures solve */
#define SBG_INST_TIMEOUT           16   /* persistent kernel hit its iteration budget */
/* Mixed form, internal: at some RHS of this instance the refinement
 * correction was larger than a set fraction of udot (1e-4 in a realize, 1e-5
 * in an integration), i.e. the FP32 factorisation of M was too poorly
 * conditioned for the mixed form's 1e-5 bar. No entry point reports it:
 * sbg_realize_acceleration recomputes such instances in FP64; a mixed batch
 * integration takes that step and the next 15 of the instance in FP64; the
 * server's mixed lane continues the request in FP64. */
#define SBG_INST_ILL_CONDITIONED   32

/* One mobilized body, numbered 1..nbodies in MobilizedBodyIndex order (Ground
 * is 0); parent < own index, as Simbody requires
 * (SimbodyMatterSubsystemRep.cpp:256-330). Transforms are 3x3 row-major
 * rotation followed by the translation: {R00,R01,R02,R10,...,R22,p0,p1,p2}.
 * Mass properties are Simbody's MassProperties(mass, com, UnitInertia) about
 * the body origin Bo, expressed in B (RigidBodyNode.h:1001-1018). */
typedef struct sbg_body_desc {
    int32_t parent;
    int32_t mobilizer;          /* sbg_mobilizer */
    double  mass;
    double  com[3];
    double  unit_inertia[6];    /* xx yy zz xy xz yz */
    double  X_PF[12];           /* inboard frame F on parent P */
    double  X_BM[12];           /* outboard frame M on body B */
    double  pitch;              /* SBG_SCREW: translation along Fz per radian about Fz (else unused) */
} sbg_body_desc;

/* Mobility force elements, applied in array order (Force.cpp:339-351, 434-443).
 *   kind 0: MobilityLinearSpring(body, MobilizerQIndex which, k=coef, q0)
 *           f[u(which)] -= k*(q[q(which)] - q0)  -- Simbody reads q[which] but
 *           writes u[which] (Force.cpp:347-350); reproduced as is.
 *   kind 1: MobilityLinearDamper(body, MobilizerUIndex which, c=coef)
 *           f[u(which)] -= c*u[which] */
typedef struct sbg_mobility_force_desc {
    int32_t kind;
    int32_t body;
    int32_t which;
    int32_t reserved;
    double  coef;
    double  q0;
} sbg_mobility_force_desc;

/* Constraint::Ball(body1, station1, body2, station2): station points fixed on
 * two bodies are held coincident (ConstraintImpl.h:1835-1993). */
typedef struct sbg_ball_constraint_desc {
    int32_t body1;
    int32_t body2;
    double  station1[3];
    double  station2[3];
} sbg_ball_constraint_desc;

/* SmoothSphereHalfSpaceForce (SmoothSphereHalfSpaceForce.cpp:252-336)
 * between a sphere fixed on a body and a half-space fixed in Ground: a
 * smoothed Hertz normal force with Hunt-Crossley dissipation and a
 * smoothed static/dynamic/viscous friction, applied at the point midway
 * through the indentation. The half-space frame is a transform in Ground
 * (its x axis is the contact normal, pointing into the half-space);
 * parameters as SmoothSphereHalfSpaceForce::setParameters, with the
 * reference's defaults when the whole parameter block is zero: stiffness 1,
 * dissipation 0, frictions 0, transition velocity 0.01, cf 1e-5, bd 300,
 * bv 50. */
typedef struct sbg_contact_desc {
    int32_t body;               /* the sphere's body, 1..nbodies */
    int32_t reserved;
    double  station[3];         /* sphere center in the body frame */
    double  radius;
    double  halfspace[12];      /* half-space frame in Ground, as the transforms above */
    double  stiffness, dissipation, static_friction, dynamic_friction, viscous_friction;
    double  transition_velocity, cf, bd, bv;
} sbg_contact_desc;

/* A whole System: matter + Force::Gravity (gravity = g * direction) +
 * mobility forces + contact spheres + Ball constraints. */
typedef struct sbg_system_desc {
    int32_t nbodies;
    int32_t nforces;
    int32_t nconstraints;
    int32_t flags;                /* SBG_SYSTEM_* bits */
    double  gravity[3];
    const sbg_body_desc*            bodies;       /* nbodies entries, body 1 first */
    const sbg_mobility_force_desc*  forces;       /* nforces entries */
    const sbg_ball_constraint_desc* constraints;  /* nconstraints entries */
    int32_t ncontacts;
    int32_t reserved2;
    const sbg_contact_desc*         contacts;     /* ncontacts entries (may be NULL when 0) */
} sbg_system_desc;

/* Integrator options (SimTKmath Integrator.h:352-383). Zero/negative fields
 * take Simbody's defaults: accuracy 1e-3, constraint tolerance accuracy/10
 * (IntegratorRep.h:737-740). */
typedef struct sbg_integ_opts {
    double  accuracy;
    double  constraint_tolerance;
    int32_t project_every_step;   /* Integrator::setProjectEveryStep */
    /* 0: the call starts with Integrator::initialize(state) (quaternions
     * normalised; with loop closures, forced position and velocity
     * projections). Nonzero: it continues the integration the previous
     * integration call on this batch left, as a second Integrator::stepTo()
     * does (AbstractIntegratorRep.cpp:341-421); SBG_ERR_STATE if the state was
     * set since or nothing has been integrated. */
    int32_t continue_integration;
} sbg_integ_opts;

/* Options of the error-controlled integrator (sbg_rk_merson_adaptive); a
 * value <= 0 takes Simbody's default. */
typedef struct sbg_adaptive_opts {
    double  accuracy;              /* Integrator::setAccuracy (1e-3) */
    double  constraint_tolerance;  /* Integrator::setConstraintTolerance (accuracy/10) */
    double  initial_step;          /* Integrator::setInitialStepSize (the timescale / 10 = 0.01) */
    double  min_step;              /* Integrator::setMinimumStepSize (none) */
    double  max_step;              /* Integrator::setMaximumStepSize (none) */
    int32_t project_every_step;    /* Integrator::setProjectEveryStep */
    int32_t max_steps;             /* accepted steps per instance before SBG_INST_TIMEOUT (1e6) */
} sbg_adaptive_opts;

typedef struct sbg_batch_config {
    int32_t precision;            /* sbg_precision */
    int32_t device;               /* CUDA device ordinal */
    int64_t device_budget_bytes;  /* 0 = no limit */
} sbg_batch_config;

typedef struct sbg_topology_s* sbg_topology;
typedef struct sbg_batch_s*    sbg_batch;

/* ---------------------------------------------------------------- library */

/* Thread-local message for the last failing call on this thread. */
const char* sbg_last_error(void);
int sbg_abi_version(void);
/* Number of CUDA devices visible (0 without a driver); never fails. */
int sbg_device_count(void);

/* --------------------------------------------------------------- topology */

/* Replaces System::realizeTopology() / SimbodyMatterSubsystemRep::endConstruction
 * (SimbodyMatterSubsystemRep.cpp:256-330): validates the system and flattens
 * it into level-ordered structure-of-arrays tables. Host only; no GPU needed. */
int sbg_topology_create(const sbg_system_desc* system, sbg_topology* out);
int sbg_topology_destroy(sbg_topology topology);
/* State sizes, as State::getNQ/getNU (State.h:962-966); levels = tree depth. */
int sbg_topology_info(sbg_topology topology, int32_t* nq, int32_t* nu,
                      int32_t* nbodies, int32_t* nlevels, int32_t* nquaternions,
                      int32_t* nconstraint_equations);
/* Simbody's default state q (quaternions = identity), u = 0
 * (RigidBodyNodeSpec_Ball.h:405-415). y gets nq+nu values. */
int sbg_topology_default_state(sbg_topology topology, double* y);

/* ------------------------------------------------------------------ batch */

/* A batch of States: instance i uses topologies[instance_topology[i]]. Device
 * memory for the whole batch is allocated here, bounded by the budget. */
int sbg_batch_create(const sbg_topology* topologies, int32_t ntopologies,
                     const int32_t* instance_topology, int32_t ninstances,
                     const sbg_batch_config* config, sbg_batch* out);
int sbg_batch_destroy(sbg_batch batch);
/* y_offsets gets ninstances+1 entries: instance i occupies
 * y[y_offsets[i] .. y_offsets[i+1]) = [q, u]; ny_total gets the total length. */
int sbg_batch_layout(sbg_batch batch, int64_t* y_offsets, int64_t* ny_total);
/* Device bytes held by the batch (state, tables and scratch). */
int sbg_batch_device_bytes(sbg_batch batch, int64_t* bytes);

/* State::setTime/updY for every instance (State.h:1027-1034). t may be NULL
 * (all zero). Copies host -> device. */
int sbg_batch_set_state(sbg_batch batch, const double* t, const double* y);
/* State::getTime/getY (State.h:962-966). Copies device -> host. */
int sbg_batch_get_state(sbg_batch batch, double* t, double* y);

/* System::realize(state, Stage::Acceleration) for every instance
 * (SimTKcommon/Simulation/include/SimTKcommon/internal/System.h:283), then
 * State::getYDot (State.h:1043-1048). ydot gets [qdot, udot] per instance in
 * the y packing; status (may be NULL) gets one SBG_INST_* word per instance.
 * Synchronous. */
int sbg_realize_acceleration(sbg_batch batch, double* ydot, int32_t* status);

/* State::updY + System::realize(state, Stage::Acceleration) +
 * State::getYDot in one call, from and to host buffers (y and ydot in the
 * batch packing; status may be NULL): the same results as
 * sbg_batch_set_state(batch, NULL, y) + sbg_realize_acceleration. For a
 * batch of one topology on the one-thread-per-instance driver, the upload,
 * realize and download run in chunks of instances on several streams so
 * that copies overlap compute (after the batch's first realize has tuned
 * it); page-locked y/ydot/status are copied directly. Synchronous. */
int sbg_realize_acceleration_host(sbg_batch batch, const double* y, double* ydot, int32_t* status);

/* SimbodyMatterSubsystem::multiplyByMInv(state, f, MInvf)
 * (Simbody/include/simbody/internal/SimbodyMatterSubsystem.h:1343):
 * f and out are packed like the u parts of y (nu values per instance). It
 * runs in the batch's precision; a mixed batch uses the FP32 recursion
 * without refinement, whose relative error grows with the condition number
 * of M. An FP64 batch gives the reference's result to 1e-12. */
int sbg_multiply_by_minv(sbg_batch batch, const double* f, double* out);

/* Tree operators on the batch's current state, for every instance. They run
 * in FP64 whatever the batch's precision and ignore the systems' own forces
 * and constraints, as the reference's do. Packing:
 *   u-like arrays (mobility forces, udot, residuals, M x, ~J F): nu values
 *     per instance, like the u parts of y;
 *   body arrays: one entry per mobilized body (Ground excluded) in the order
 *     of the system description's bodies, instances one after another
 *     (nbodies entries each). A SpatialVec entry is 6 values (angular then
 *     linear: moment and force, or angular and linear velocity /
 *     acceleration), expressed in Ground at the body origin. A spatial
 *     inertia entry is 10 values: mass, the mass center measured from the
 *     body origin (3), and the unit inertia about the body origin (xx yy zz
 *     xy xz yz), all in Ground.
 * status (may be NULL) gets one SBG_INST_* word per instance (NONFINITE for
 * a non-finite result). Synchronous. */

/* SimbodyMatterSubsystem::calcResidualForceIgnoringConstraints(state,
 * appliedMobilityForces, appliedBodyForces, knownUdot, residualMobilityForces)
 * (Simbody/include/simbody/internal/SimbodyMatterSubsystem.h:2234):
 * residual = M udot + C(q,u) - f_applied - ~J F_applied (inverse dynamics,
 * Stage::Velocity). Any of the three inputs may be NULL: all zero, as a
 * zero-length Vector is for the reference. */
int sbg_calc_residual_force(sbg_batch batch, const double* mobility_forces, const double* body_forces,
                            const double* known_udot, double* residual, int32_t* status);
/* SimbodyMatterSubsystem::multiplyByM(state, a, Ma) (SimbodyMatterSubsystem.h:1262). */
int sbg_multiply_by_m(sbg_batch batch, const double* a, double* Ma, int32_t* status);
/* SimbodyMatterSubsystem::multiplyBySystemJacobian(state, u, Ju)
 * (SimbodyMatterSubsystem.h:554): Ju is a body array of SpatialVecs. */
int sbg_multiply_by_system_jacobian(sbg_batch batch, const double* u, double* Ju, int32_t* status);
/* SimbodyMatterSubsystem::multiplyBySystemJacobianTranspose(state, F_G, f)
 * (SimbodyMatterSubsystem.h:646): F_G is a body array of SpatialVecs. */
int sbg_multiply_by_system_jacobian_transpose(sbg_batch batch, const double* F_G, double* f, int32_t* status);
/* SimbodyMatterSubsystem::calcCompositeBodyInertias(state, R)
 * (SimbodyMatterSubsystem.h:2323): R is a body array of spatial inertias. */
int sbg_calc_composite_body_inertias(sbg_batch batch, double* R, int32_t* status);
/* Device time in milliseconds of the kernels of the batch's last tree
 * operator call (its copies excluded), from CUDA events on the batch's stream. */
int sbg_batch_last_operator_ms(sbg_batch batch, double* ms);
/* Mixed batches: how many instance realizations so far were recomputed in
 * FP64 because the refinement reported an ill-conditioned M (see
 * SBG_INST_ILL_CONDITIONED); 0 for other precisions. Synchronous. */
int sbg_batch_fallback_count(sbg_batch batch, int64_t* n);
/* Mixed batches: how many instance steps of the batch's integrations so far
 * were taken in FP64 because a mixed RHS of the step met an ill-conditioned M
 * (the step itself and the instance's next 15); 0 for other precisions. No
 * counterpart in the reference. Synchronous. */
int sbg_batch_fp64_steps(sbg_batch batch, int64_t* n);

/* RungeKuttaMersonIntegrator with setFixedStepSize(h), initialize(state) and
 * exactly nsteps internal steps of h (stepTo looped with
 * setReturnEveryInternalStep; RungeKuttaMersonIntegrator.cpp:86-140,
 * AbstractIntegratorRep.cpp:137-207, 341-577), for every instance, on the
 * batch's current device state, which is advanced in place. status (may be
 * NULL) gets the OR of SBG_INST_* words per instance. opts may be NULL; with
 * opts->continue_integration the call continues the previous one. */
int sbg_rk_merson_fixed(sbg_batch batch, double h, int32_t nsteps,
                        const sbg_integ_opts* opts, int32_t* status);
/* Integrator::stepTo(t_report) of a fixed-step RungeKuttaMersonIntegrator
 * with setAllowInterpolation(false), so tMax = t_report
 * (AbstractIntegratorRep.cpp:229-240): every instance steps from its current
 * time; each step ends at t0 + h unless t_report lies within 0.95 h (a
 * shortened last step) or within 1.001 h (t_report itself) of t0
 * (AbstractIntegratorRep.cpp:536-544). An instance already at t_report does
 * not move. Without opts->continue_integration the call begins with
 * Integrator::initialize; with it, stepTo(0.5) then stepTo(1.0) gives the
 * reference's two-call trajectory. SBG_INST_TIMEOUT if time stops advancing. */
int sbg_rk_merson_step_to(sbg_batch batch, double h, double t_report,
                          const sbg_integ_opts* opts, int32_t* status);

/* State::getQDotDot() at Stage::Acceleration (SimbodyMatterSubsystem
 * calcQDotDot over the mobilizers): Pin/Slider/Universal qdotdot = udot; a
 * Ball or Free quaternion gets N(q) udot_w + NDot(q,qdot) w computed as
 * Rotation::convertAngVelDotToQuaternionDotDot (RigidBodyNodeSpec_Ball.h:355-390,
 * RigidBodyNodeSpec_Free.h:418-455, Rotation.h:1006-1013), a Free body's
 * translation its udot. qdotdot gets nq values per instance, back to back in
 * instance order. Formed from the state and the udot of the last realize,
 * which must be of the current state (SBG_ERR_STATE otherwise). Synchronous. */
int sbg_batch_get_qdotdot(sbg_batch batch, double* qdotdot);

/* Error-controlled RungeKuttaMersonIntegrator: setFinalTime(t_final),
 * initialize(state) (quaternions normalized) and stepTo(t_final) for every
 * instance of an FP64 batch without loop closures, each with its own step
 * size (AbstractIntegratorRep.cpp:341-577: takeOneStep, attemptDAEStep's
 * projection, adjustStepSize :448-502). stats (may be NULL) gets the accepted
 * and rejected steps of each instance (2 values per instance). Synchronous.
 * SBG_ERR_UNSUPPORTED for mixed batches and loop closures. */
int sbg_rk_merson_adaptive(sbg_batch batch, double t_final, const sbg_adaptive_opts* opts, int32_t* status,
                           int64_t* stats);

/* ------------------------------------------- device-resident (timing) path */

/* The batch's CUDA stream, as a cudaStream_t cast to void*. */
void* sbg_batch_stream(sbg_batch batch);
/* realize(Acceleration) on the resident state; ydot stays on the device.
 * Asynchronous on the batch stream. */
int sbg_realize_acceleration_async(sbg_batch batch);
/* RK Merson on the resident state, asynchronous on the batch stream. */
int sbg_rk_merson_fixed_async(sbg_batch batch, double h, int32_t nsteps,
                              const sbg_integ_opts* opts);
/* sbg_rk_merson_step_to, asynchronous on the batch stream. */
int sbg_rk_merson_step_to_async(sbg_batch batch, double h, double t_report,
                                const sbg_integ_opts* opts);
/* Copy the resident ydot / status of the last realize to host (synchronous). */
int sbg_batch_get_ydot(sbg_batch batch, double* ydot, int32_t* status);
int sbg_batch_sync(sbg_batch batch);
/* Number of kernel launches issued by this batch since creation. */
int64_t sbg_batch_launch_count(sbg_batch batch);
/* Occupancy variant the batch's tuner picked for its FP32 kernels (1 = two
 * 128-thread blocks per SM, 4 = four, 7 = seven 64-thread blocks per SM for
 * the one-thread-per-instance segment), 0 before the first realize or
 * integration, -1 for a null batch. No counterpart in the reference. */
int sbg_batch_kernel_variant(sbg_batch batch);
/* Lanes-per-tree setting the tuner picked for the batch's level-parallel
 * segment (lanes = next power of two of the widest level, shifted right by
 * this), -1 for a null batch. No counterpart in the reference. */
int sbg_batch_group_lanes_shift(sbg_batch batch);

/* ----------------------------------------------------------------- serving */

/* No counterpart in the reference (Simbody runs one Integrator per State on
 * the calling thread). A server admits rollout requests -- one State of any
 * supported System, Integrator::initialize(state) and fixed-step RK-Merson
 * stepTo(t0 + nsteps*h), as sbg_rk_merson_fixed does for one instance --
 * and runs them with continuous batching on one GPU: every tick, each
 * resident request advances by min(its chunk, remaining) steps in the same
 * kernel launch as all other resident requests; finished requests leave
 * after their tick and queued ones (strict arrival order) take their slots
 * and memory. The server allocates its whole device budget once, at
 * creation (device arena split into table, state and scratch pools); a
 * request is admitted only while its share fits. The server runs three
 * lanes, each with its own share of the budget and slots and its own tick
 * cadence, so that requests never wait on much costlier ones: lane 0 the
 * trees without loop closures (the server's precision), lanes 1 and 2 in
 * FP64 the trees with loop closures, split by estimated cost per step.
 * A mixed-precision request that fails is rerun from its initial state in
 * FP64 (sbg_request_info.attempts). A request's result does not depend on
 * which other requests share its ticks. */
typedef struct sbg_server_s* sbg_server;

typedef struct sbg_server_config {
    int32_t precision;            /* sbg_precision of the tree recursions; loop
                                     closures always run in FP64 */
    int32_t device;               /* CUDA device ordinal */
    int64_t device_budget_bytes;  /* device memory the server holds (> 0) */
    int32_t max_slots;            /* resident requests at most (0 = 65536; >= 3) */
    int32_t chunk_steps;          /* RK steps per tick of a request of median
                                     cost (0 = 64); each request's own chunk
                                     scales with the inverse of its estimated
                                     GPU time per step (1 .. 16x) */
} sbg_server_config;

typedef struct sbg_request_info {
    int32_t done;       /* 1 once the final state is on the host */
    int32_t status;     /* OR of the SBG_INST_* words of its steps */
    int32_t nbodies;
    int32_t nsteps;
    double  t;          /* final time */
    double  submit_s;   /* server clock (sbg_server_clock) at submission, */
    double  admit_s;    /* at admission (-1 while queued) and */
    double  done_s;     /* when the result reached the host (-1 before) */
    int32_t attempts;   /* 2: the mixed-precision run failed (non-finite, singular
                           D or failed projection) and the request was rerun
                           from its initial state in FP64 */
    int32_t fp64_steps; /* 1: a mixed-precision request reached a state where
                           the mixed form's refinement could not meet its bar
                           (SBG_INST_ILL_CONDITIONED): that RHS and the next
                           16 steps ran in FP64, then the mixed form was
                           tried again */
} sbg_request_info;

typedef struct sbg_server_stats {
    int64_t submitted, completed, queued, resident, peak_resident;
    int64_t ticks, launches;
    int64_t body_steps;          /* sum of bodies x steps of completed requests */
    int64_t device_bytes;        /* device memory held (the arena) */
    int32_t max_slots, chunk_steps;
    int64_t pool_capacity[5];    /* rows, forces, state, scratch, loop scratch */
    int64_t pool_in_use[5];
    double  gpu_seconds;         /* GPU time of the completed ticks (copies + kernels) */
    double  host_seconds;        /* host time in sbg_server_tick, not counting waits for the GPU */
} sbg_server_stats;

int sbg_server_create(const sbg_server_config* config, sbg_server* out);
int sbg_server_destroy(sbg_server server);
/* Queue a request (host only, never waits for the GPU; thread-safe). The
 * topology is copied: it may be destroyed after the call. y0 has nq+nu
 * values. SBG_ERR_BUDGET if the request could never fit the server. */
int sbg_server_submit(sbg_server server, sbg_topology topology, const double* y0, double t0, double h,
                      int32_t nsteps, const sbg_integ_opts* opts, int64_t* request_id);
/* One scheduling round: collect finished ticks, admit, launch one chunk of
 * every resident request. Returns without waiting when the previous tick is
 * still running (at most two ticks are in flight). ncompleted (may be NULL)
 * gets the number of requests whose results arrived during this call. */
int sbg_server_tick(sbg_server server, int32_t* ncompleted);
/* Tick until every submitted request has its result on the host. */
int sbg_server_drain(sbg_server server);
/* Result of a request: y (nq+nu values, may be NULL) once info->done; with
 * info given, an unfinished request returns SBG_OK and done = 0. */
int sbg_server_result(sbg_server server, int64_t request_id, double* y, sbg_request_info* info);
int sbg_server_get_stats(sbg_server server, sbg_server_stats* stats);
/* The same for one lane: 0 = trees, 1 / 2 = FP64 lanes (loop closures and
 * reruns; cheaper / costlier per step). */
int sbg_server_get_lane_stats(sbg_server server, int32_t lane, sbg_server_stats* stats);
/* Seconds since the server was created: the clock of sbg_request_info. */
double sbg_server_clock(sbg_server server);
/* The admission and chunk policy run without a device (for checking it):
 * request i has footprint units[5*i .. 5*i+5) in the pools of `capacity`
 * (rows, forces, state, scratch, loop scratch), horizon horizons[i], and
 * arrives at tick arrival_tick[i] (non-decreasing). admit_tick / done_tick
 * get the tick of its admission and of its last chunk. */
int sbg_serve_simulate(int32_t n, const int64_t* units, const int32_t* horizons, const int64_t* arrival_tick,
                       const int64_t* capacity, int32_t max_slots, int32_t chunk_steps, int64_t* admit_tick,
                       int64_t* done_tick, int64_t* peak_resident);

/* ------------------------------------------------ allocation-free realize */

/* No counterpart in the reference: an addition for callers that may not
 * allocate device memory (a control loop that allocates only at start-up, a
 * host framework that hands out device buffers from its own pool). It runs
 * the plain FP64 realize(Stage::Acceleration) for ninstances states of ONE
 * topology with no cudaMalloc/cudaFree: the caller passes device buffers
 *   y      ninstances * (nq+nu) doubles, [q, u] per instance, back to back
 *   ydot   same size, receives [qdot, udot]
 *   status ninstances SBG_INST_* words
 * and the per-body scratch lives in a 16 MiB file-scope device array (the
 * topology tables in fixed device arrays: at most 256 bodies and 4096
 * mobility-force elements); larger topologies are rejected with
 * SBG_ERR_INVALID, and ones with loop closures or contact spheres with
 * SBG_ERR_UNSUPPORTED. Runs asynchronously on `stream` (a cudaStream_t, NULL =
 * default stream) of the current device. The first call on a device does the
 * set-up: it looks up the arrays' device addresses (cudaGetSymbolAddress), and
 * with CUDA's lazy module loading that is also when the driver loads this
 * module and creates its fixed arrays (about 16.3 MiB), so that first call can
 * fail with SBG_ERR_CUDA if the device has no memory left. Make it at start-up;
 * later calls allocate nothing. Each call uploads the topology tables from
 * host memory that ends with the call, so a call on a stream that is being
 * captured returns SBG_ERR_UNSUPPORTED. All calls share
 * the arrays, which keep the last call's contents: calls that overlap on the
 * GPU race. Message of the last failure: sbg_noalloc_last_error(). */
int sbg_realize_acceleration_noalloc(sbg_topology topology, int32_t ninstances,
                                     const double* y, double* ydot,
                                     int32_t* status, void* stream);
const char* sbg_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SIMBODY_GB300_H_ */
