// topology_internal.h -- the host-side flattened topology behind the opaque
// sbg_topology handle (shared by capi.cpp and k_noalloc.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/simbody_gb300.h"
#include "engine.h"

// A flattened topology: bodies in level order (the reference's rbNodeLevels).
struct sbg_topology_s {
    int nb = 0, nq = 0, nu = 0, nlevels = 0, nquat = 0, ncons = 0;
    int maxNonFreeDof = 0;
    int64_t recSize = 0;                 // scratch elements per instance
    std::vector<int32_t> parent, info, qoff, uoff, srec, fbeg, fcnt;
    std::vector<int32_t> bodyOfRow;             // descriptor index (0-based) of each row
    std::vector<int32_t> levStart;              // nlevels + 1 local rows
    std::vector<int32_t> cbeg, ccnt, clist;     // children (local rows) per row
    int maxLevelWidth = 0;
    bool chain = false;                         // every row's parent is the previous row
    std::vector<double> par;             // kParamStride per row
    std::vector<int32_t> fkw;            // force elements, grouped by row
    std::vector<double> fcoef, fq0;
    std::vector<int32_t> kbeg, kcnt;     // contact spheres per row: offset in kpar, count
    std::vector<double> kpar;            // kContactStride per contact
    int ncontacts = 0;
    double gravity[3] = {0, 0, 0};
    std::vector<double> defaultY;
    std::vector<sbg_ball_constraint_desc> cons;
    // loop closures in local rows: body 1, body 2 (-1 = Ground) and the
    // stations (station 1, station 2); slot index per row (-1 = none)
    std::vector<int32_t> lcons, lslot;
    std::vector<double> lst;
    int nslots = 0;
};

namespace sbg {
// Records msg as the calling thread's sbg_last_error() message; returns code.
int setError(int code, const std::string& msg);
}  // namespace sbg

// Scratch-record offsets of the rows of `t` when every non-Free row is given
// the record of an nm-mobility body (Free rows keep 6): lanes of a warp that
// process the same row of different topologies then address the same record
// elements. *total gets the record length of one instance.
inline std::vector<int32_t> paddedRecords(const sbg_topology_s& t, int nm, int64_t* total) {
    std::vector<int32_t> off(t.nb);
    int64_t rec = 0;
    for (int r = 0; r < t.nb; ++r) {
        const int n = (t.info[r] >> 4) & 15;
        off[r] = (int32_t)rec;
        rec += sbg::scratchRecordSize(n == 6 ? 6 : nm);
    }
    if (total) *total = rec;
    return off;
}

// Field-major record length of the level-parallel layout: every row gets the
// widest record of the instance (6 columns if any row is Free, else nm).
inline int64_t rowsRecordWidth(const sbg_topology_s& t, int nm) {
    int w = nm;
    for (int r = 0; r < t.nb; ++r)
        if (((t.info[r] >> 4) & 15) == 6) w = 6;
    return sbg::scratchRecordSize(w);
}

