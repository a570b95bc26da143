// topology_internal.h -- the host-side flattened topology behind the opaque
// sbg_topology handle (shared by capi.cpp and k_noalloc.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/simbody_gb300.h"
#include "engine.h"

// A flattened topology: bodies in level order (the reference's rbNodeLevels).
struct sbg_topology_s {
    int nb = 0, nq = 0, nu = 0, nlevels = 0, nquat = 0, ncons = 0;
    int maxNonFreeDof = 0;
    int64_t recSize = 0;                 // scratch elements per instance
    std::vector<int32_t> parent, info, qoff, uoff, srec, fbeg, fcnt;
    std::vector<double> par;             // kParamStride per row
    std::vector<int32_t> fkw;            // force elements, grouped by row
    std::vector<double> fcoef, fq0;
    double gravity[3] = {0, 0, 0};
    std::vector<double> defaultY;
    std::vector<sbg_ball_constraint_desc> cons;
};

