// engine.h -- device-side table layout shared by the host runtime (capi.cpp)
// and the CUDA kernels (abi_device.cuh and the k_*.cu instantiations).
//
// HBM layout of a batch
//   Body table (one row per mobilized body of every distinct topology, bodies
//   of a topology stored in level order, i.e. the rbNodeLevels order of
//   SimbodyMatterSubsystemRep.cpp:256-330):
//     parent  local row of the parent body within its topology, -1 = Ground
//     info    mobilizer | ndof << 4
//     qoff/uoff  Simbody q/u slot of the body (body-index order)
//     srec    offset of the body's scratch record within its instance record
//     fbeg/fcnt  mobility-force elements of this body, in application order
//     par     kParamStride parameters per body (AoS): mass, com[3],
//             unit inertia[6] (xx yy zz xy xz yz), R_PF[9], p_PF[3],
//             R_MB[9], p_MB[3], screw pitch; stored in FP64 and, for the
//             mixed form, FP32.
//   Instance table: first body row, body count, q/u sizes, addressing of its
//   state column and scratch record, gravity index.
//   State y, derivatives and scratch are "columns": element k of instance i
//   lives at base_i + k*stride_i. A group of instances that share one
//   topology uses stride = ninstances (structure of arrays: a warp's loads of
//   element k coalesce); instances with their own topology use stride 1
//   (each thread walks its own contiguous record).
#pragma once
#include <cstdint>

namespace sbg {

constexpr int kParamStride = 35;
constexpr int kMaxDof = 6;

// Scratch record of one body (elements of the arithmetic type R), n = ndof:
//   0  R_GB[9] p_GB[3] V_GB[6]  kinematics (only for children that are not the
//                               next row); pass 3 reuses [0,6) for A_GB and,
//                               in the mixed form, [6,18) for A in double-float
//  18  pc[3] Gi[6] l[3] a[6] bF[6]
//  42  Pacc: M[6] J[6] F[9], zacc[6]      (pass 2 accumulators)
//      reused after pass 2: [42,54) F_df (double-float inverse-dynamics force),
//      [54,60) z2acc (refinement M^-1 accumulator); the tree operators
//      (ops_device.cuh) keep A [42,48) and F [48,54), or a composite inertia
//      [42,52), there
//  69  H[6n] f[n] DI[n*n] G[6n] eps[n] udot0[n]
#ifdef __CUDACC__
#define SBG_HD __host__ __device__
#else
#define SBG_HD
#endif
SBG_HD constexpr int scratchRecordSize(int n) { return 69 + 15 * n + n * n; }
constexpr int kRecKin = 0, kRecPc = 18, kRecGi = 21, kRecL = 27, kRecA = 30, kRecBF = 36, kRecPacc = 42,
              kRecZacc = 63, kRecH = 69, kRecFdf = 42, kRecZ2acc = 54;

// Body-table info word: mobilizer | ndof << 4 | flags.
enum : int {
    F_RPF_I = 1 << 8,      // R_PF is the identity
    F_RMB_I = 1 << 9,      // R_BM is the identity
    F_PMB_0 = 1 << 10,     // p_BM is zero
    F_PPF_0 = 1 << 11,     // p_PF is zero
    F_CARRY = 1 << 12,     // the parent is the previous row: values travel in registers
    F_MEMCHILD = 1 << 13,  // some child is not the next row: it reads/accumulates through the record
    F_LOOPBODY = 1 << 14,  // body 1 or 2 of a Ball loop closure: keeps a slot record
    F_LOOPPATH = 1 << 15,  // a loop body or an ancestor of one: the only rows a unit
                           // constraint force reaches on its way to the base
    F_QUAT = 1 << 16,      // Ball or Free with quaternion coordinates (not Euler angles)
    F_CONTACT = 1 << 17,   // carries SmoothSphereHalfSpaceForce spheres (kbeg/kcnt)
};

// Loop closures (Constraint::Ball), FP64 only. Each body named
// by a constraint has a slot record after the body records of its instance:
//   0  R_GB[9] p_GB[3] V_GB[6]   from the position/velocity pass
//  18  A_GB[6]                   tree acceleration (pass 3)
//  24  B[6]                      result of a unit-force sweep (acceleration
//                                or velocity of the body origin)
//  30  F[6]                      applied spatial force (torque, force) at Bo
//  36  B[6] x 2, F[6] x 2         columns 1 and 2 of a three-column Gram sweep
constexpr int kSlotA = 18, kSlotB = 24, kSlotF = 30, kSlotB3 = 36, kSlotF3 = 48, kSlotSize = 60;
constexpr int kMaxLoopCons = 4;             // Ball constraints per instance
constexpr int kMaxLoopEq = 3 * kMaxLoopCons;
constexpr int F_MEMACC = F_MEMCHILD;

// Warp tile of the shared-topology scratch layout.
constexpr int kTile = 32;

struct DevTables {
    const int32_t* parent;
    const int32_t* info;
    const int32_t* qoff;
    const int32_t* uoff;
    const int32_t* srec;
    const int32_t* fbeg;
    const int32_t* fcnt;
    const double* par64;
    const float* par32;
    const int32_t* fkind_which;  // kind << 8 | which
    const double* fcoef64;
    const double* fq064;
    const float* fcoef32;
    const float* fq032;
    // per instance
    const int32_t* ibody;    // first body row
    const int32_t* inb;      // number of bodies
    const int32_t* inq;
    const int32_t* inu;
    const int64_t* ybase;    // state column base
    const int64_t* ystride;
    const int64_t* sbase;    // scratch column base
    const int64_t* sstride;
    const double* grav;      // per instance gravity (3)
    const int32_t* order;    // position -> instance (chain segment first, then group segment)
    int32_t ninst;
    // level-parallel (group) driver
    const int32_t* ilev;     // per instance: first entry of its level table in levStart
    const int32_t* inlev;    // per instance: number of levels
    const int32_t* levStart; // per topology: local row where each level starts (+ end)
    const int32_t* cbeg;     // per body row: first child in clist
    const int32_t* ccnt;     // per body row: number of children
    const int32_t* clist;    // children as local rows
    const int32_t* blkFirst; // per group block: first order position (+ end)
    const int32_t* blkG;     // per group block: lanes per instance
    // loop closures
    const int32_t* lrec;     // per body row: slot record offset, -1 if none
    const int32_t* lcons;    // per constraint: local row of body 1, of body 2 (-1 = Ground)
    const double* lst;       // per constraint: station 1 (in body 1), station 2 (in body 2)
    const int32_t* lslot;    // per body row: slot index of a loop body (-1 = none): level-parallel layout
    const int32_t* bidx;     // per body row: index of the body in its system description (tree operators)
    // FP64 mirror of the scratch with the same element offsets (mixed batches
    // and the server's mixed lane; null otherwise): where the mixed form's
    // refinement reports an ill-conditioned M the RHS is recomputed in FP64
    // on these records.
    double* scratch64;
    unsigned long long* fallbacks;  // instances recomputed in FP64 by realize (cumulative; null = none)
    const int32_t* icons;    // per instance: first constraint
    const int32_t* incons;   // per instance: number of constraints
    // per-instance integration control (the serving loop; null in a batch,
    // whose instances share the launch's step count, step size and options)
    const int32_t* ictl;     // steps of this launch | kCtl* flags
    const double* iparam;    // h, accuracy, constraint tolerance (3 per instance)
    // One-step launches of a mixed batch integration (null otherwise). At
    // launch L an instance is in FP64 mode when fbMode[(L & 1) * ninst + i]
    // is set: the FP64 list kernel steps it (it is on fbList[L & 1], length
    // fbCount[L & 1]) while the mixed kernels, concurrently, step the others.
    // Each launch's owner of an instance writes its mode for launch L + 1 and
    // puts it on the next list if FP64. An instance whose mixed step meets an
    // ill-conditioned M leaves its state as it was (it falls one step behind)
    // and takes that step and the next kFp64Steps - 1 in FP64 (fbLeft counts
    // them). stepsLeft counts the steps an instance still has to take in a
    // fixed-count call (null for stepTo).
    int32_t* fbList;         // 2 x ninst
    int32_t* fbCount;        // 2
    int32_t* fbMode;         // 2 x ninst
    int32_t* fbLeft;         // per instance
    int32_t* stepsLeft;      // per instance
    double* fbuf64;          // FP64 stage derivatives of the FP64-mode instances (4 planes)
    unsigned long long* fbSteps;  // FP64 steps taken by the list kernel (cumulative)
    // Contact spheres on a ground half-space (SmoothSphereHalfSpaceForce),
    // grouped by body row in element order; read only for F_CONTACT rows
    // (null where no topology has any).
    const int32_t* kbeg;     // per body row: offset of its first contact's values in kpar
    const int32_t* kcnt;     // per body row: number of contacts
    const double* kpar64;    // kContactStride per contact
    const float* kpar32;
};
// Per-contact parameters: station[3] (body frame), radius, contact normal
// n[3] (the half-space frame's x axis in Ground), surface point p_H[3] (its
// origin in Ground), Hertz factor (4/3) k sqrt(r k) with k = stiffness^(2/3)/2,
// dissipation c, static, dynamic and viscous friction, transition velocity,
// cf, bd, bv, 2/(3c) (infinite when c = 0).
constexpr int kContactStride = 20;
// FP64 steps an instance takes, from the step whose mixed RHS met an
// ill-conditioned M, before it tries the mixed form again.
constexpr int kFp64Steps = 16;
// Lanes per instance of the FP64 list kernel (level-parallel driver).
constexpr int kFbLanes = 8;
constexpr int kCtlSteps = (1 << 24) - 1;
constexpr int kCtlInit = 1 << 30;                // first launch: Integrator::initialize projections
constexpr int kCtlProjectEveryStep = 1 << 29;    // Integrator::setProjectEveryStep(true)
// Status-word bits kept across a request's launches in the server
// (stripped before the status is reported): its RHS runs in FP64 for the
// next kStFp64Left steps (a count in bits 20-27), after which it tries the
// mixed form again; kStWasFp64 records that it ever switched.
constexpr int kStFp64 = 1 << 30;
constexpr int kStWasFp64 = 1 << 29;
constexpr int kStFp64LeftShift = 20;
constexpr int kStFp64LeftMask = 0xFF << kStFp64LeftShift;
// The mixed form's refinement trusts its FP32 factorisation while the
// correction stays within this fraction of udot (max-norms): 1e-4 in a
// realize, where a flagged instance costs an FP64 recomputation after the
// mixed pass, and 1e-5 in an integration (batch steps and the server), whose
// FP64 steps overlap the mixed ones.
constexpr float kIllConditioned = 1e-4f;
constexpr float kIllConditionedStep = 1e-5f;

// How one batch operation is launched: order positions [0, nChain) run the
// chain driver (one thread per instance, width nm), the next nLoop positions
// the FP64 chain driver with loop closures, and nGroupBlocks blocks of the
// level-parallel driver cover the rest.
struct LaunchPlan {
    int nChain;
    int nGroupBlocks;
    int nm;
    int variant;  // 1: registers as needed; 4: at most 128 registers (FP32 only); 7: 64-thread blocks; 8: 7 staged (realize)
    int nLoop;    // order positions [nChain, nChain + nLoop): instances with loop closures (FP64 chain driver)
    int chainFirst;  // first order position of the chain segment launch (a sub-range of it: pipelined realize)
    int groupFirst;  // first block of the level-parallel launch in the block table
    int nLoopGroupBlocks;  // blocks [loopGroupFirst, +n): loop-closure instances on the level-parallel driver (FP64)
    int loopGroupFirst;
};

}  // namespace sbg
