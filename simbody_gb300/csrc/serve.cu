// serve.cu -- the serving loop: continuous batching of rollout requests of
// different topologies and horizons on one GPU (sbg_server_* in
// include/simbody_gb300.h).
//
// A request is Integrator::initialize(state) followed by fixed-step
// RK-Merson stepTo(t0 + n h) for one System (RungeKuttaMersonIntegrator.cpp:
// 86-140, AbstractIntegratorRep.cpp:137-207, 341-577). The server keeps every
// admitted request resident in a device arena that it allocates once, at
// creation, to the size of its budget:
//   rows pool      body tables (parent, mobilizer info, q/u slots, records,
//                  forces, children, levels) and the FP64/FP32 parameters
//   forces pool    mobility-force elements
//   state pool     y = [q, u] (FP64) and the four RK stage planes
//   scratch pools  per-body records of the level-parallel driver, in the
//                  server's precision and (loop closures) in FP64
//   slots          per-request instance entries (the DevTables' instance
//                  arrays), max_slots of them
// Each tick (sbg_server_tick) the host
//   1. reads back the results of finished ticks,
//   2. admits queued requests, in arrival order, while a slot and room in
//      every pool are free,
//   3. plans one chunk (min(chunk_steps, remaining) steps) for every
//      resident request,
//   4. enqueues on the server's stream: one host->device copy of a staging
//      buffer (new requests' tables and states, this tick's control arrays),
//      a copy kernel that scatters it into the arena, the RK-Merson kernels
//      (level-parallel driver for the trees on a side stream, forked and
//      joined; FP64 level-parallel driver with the multiplier solve for the
//      loop closures), a copy kernel that gathers the finished requests'
//      states, and one device->host copy of them.
// Requests that arrive while others are on the GPU join at the next tick,
// into the slots and memory that finished requests gave back. A request's
// arithmetic depends only on its own tables and state: the RK kernels carry
// nothing between launches except y, t and the status word, so the chunking
// and the company a request keeps do not change its result.
#include "../../include/simbody_gb300.h"
#include "engine.h"
#include "kernels.h"
#include "serve_sched.h"
#include "topology_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <string>
#include <unordered_map>
#include <vector>

namespace sbg {

// One copy of `words` 4-byte words; src and dst are device addresses.
struct CopyDesc {
    uint64_t src, dst;
    uint32_t words, pad;
};

__global__ void copyWordsKernel(const CopyDesc* __restrict__ d, int n) {
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const CopyDesc c = d[i];
        const uint32_t* s = reinterpret_cast<const uint32_t*>(c.src);
        uint32_t* t = reinterpret_cast<uint32_t*>(c.dst);
        for (uint32_t w = threadIdx.x; w < c.words; w += blockDim.x) t[w] = s[w];
    }
}

static cudaError_t launchCopies(const CopyDesc* d, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    copyWordsKernel<<<std::min(n, 4096), 128, 0, s>>>(d, n);
    return cudaGetLastError();
}

}  // namespace sbg

using namespace sbg;

namespace {

// Lanes per request: G = pow2ceil(widest level) >> shift, in [2, 32].
int lanesShift() {
    static const int shift = [] {
        const char* v = std::getenv("SBG_SERVE_LANES_SHIFT");  // tuning override
        return v ? std::max(0, std::min(3, std::atoi(v))) : 0;  // all lanes: latency over throughput
    }();
    return shift;
}

int groupLanes(const sbg_topology_s& t) {
    int w = 1;
    while (w < t.maxLevelWidth) w <<= 1;
    return std::max(2, std::min(32, w >> lanesShift()));
}

// Relative GPU time of one RK-Merson step of a request, in serial body
// visits per RHS on its driver:
//   level-parallel driver  sum over levels of ceil(width / lanes)
//   loop closures          the same tree passes in FP64, plus the loop-path
//                          rows of the 2m+1 constraint sweeps and the
//                          all-body correction, run on one lane
// A request's steps per tick are the server's chunk scaled by
// kRefCost / cost, so that every request's chunk takes about the same time
// and no request waits on a slower neighbour.
constexpr double kRefCost = 8.0;          // the median request of the uneven-tree distribution
constexpr double kLoopDriverWeight = 3.0;  // FP64 lanes vs. FP32 lanes
double stepCost(const sbg_topology_s& t, bool loops, int G) {
    if (!loops) {
        double slots = 0;
        for (int L = 0; L < t.nlevels; ++L) slots += (t.levStart[L + 1] - t.levStart[L] + G - 1) / G;
        return slots;
    }
    double slots = 0;
    for (int L = 0; L < t.nlevels; ++L) slots += (t.levStart[L + 1] - t.levStart[L] + G - 1) / G;
    int path = 0;
    for (int r = 0; r < t.nb; ++r) path += (t.info[r] & F_LOOPPATH) != 0;
    const int m = 3 * t.ncons;
    return kLoopDriverWeight * (slots + (double)path * (2 * m + 1) / 3.0 + t.nb / 3.0);
}

// Units of the pools per body row of a typical request (a tree of
// 4..256 bodies with a Free root, Pin/Slider/Universal/Ball children, a
// spring and a damper per mobility, 20% with loop closures): how the
// budget is split between the pools.
constexpr double kUnitsPerRow[kNumPools] = {1.05, 4.0, 8.0, 200.0, 64.0};
constexpr int64_t kAlign[kNumPools] = {1, 1, 2, 32, 2};

struct ServeReq {
    int64_t id = 0;
    int32_t sched = -1;          // index in the scheduler's table
    bool loops = false;
    int32_t G = 2;
    int nb = 0, nq = 0, nu = 0, nlevels = 0, nf = 0, ncons = 0;
    int64_t recW = 0;            // record width of the level-parallel layout
    double t0 = 0, h = 0, acc = 1e-3, ctol = 1e-4;
    bool pes = false;
    double grav[3] = {0, 0, 0};
    // host image of the device tables (request-relative)
    std::vector<int32_t> rowsI;  // 12 int32 tables x (nb + 1) rows, table-major
    std::vector<double> par64;   // kParamStride x nb
    std::vector<int32_t> fkw;
    std::vector<double> fcoef, fq0;
    std::vector<double> kpar;    // contact spheres: kContactStride values each, after the forces in the force pool
    std::vector<int32_t> lcons;  // 2 per constraint (local rows)
    std::vector<double> lst;     // 6 per constraint
    std::vector<double> y0;
    // result
    std::vector<double> y;
    double t = 0;
    int32_t status = 0;
    bool done = false;
    double submitS = 0, admitS = -1, doneS = -1;
    int64_t steps = 0;
    Footprint fp;
    double cost = 0;       // estimated GPU time per step (stepCost)
    int32_t attempts = 1;  // 2: rerun in FP64 after the mixed-precision run failed
    int32_t fp64Steps = 0; // 1: its RHS switched to FP64 (an ill-conditioned M)
};

enum RowTable { R_PARENT = 0, R_INFO, R_QOFF, R_UOFF, R_SREC, R_FBEG, R_FCNT, R_LREC, R_CBEG, R_CCNT, R_CLIST, R_LEV,
                R_LSLOT, R_KBEG, R_KCNT, kRowTables };

struct TickRec {
    int parity = 0;
    std::vector<std::pair<int64_t, int64_t>> results;  // (request id, offset in the result buffer, in words)
};

}  // namespace

struct ServeLane {
    int precision = SBG_PRECISION_MIXED, device = 0;
    int64_t budget = 0;
    int32_t maxSlots = 0, chunk = 64;
    size_t rsz = 4;
    Scheduler sched;
    int64_t cap[kNumPools] = {};
    std::vector<void*> bufs;
    int64_t devBytes = 0;
    DevTables T{};
    // arena
    int32_t* rowsI[kRowTables] = {};
    double* par64 = nullptr;
    float* par32 = nullptr;    // null in an FP64 server
    int32_t* fkw = nullptr;
    double *fcoef64 = nullptr, *fq064 = nullptr;
    float *fcoef32 = nullptr, *fq032 = nullptr;
    double* y = nullptr;
    void* fbuf = nullptr;
    void* fbufLoop = nullptr;
    void* scratch = nullptr;
    double* scratch64 = nullptr;  // mixed lane: FP64 mirror of scratch (same offsets)
    double* scratchLoop = nullptr;
    // slots
    int32_t *ibody = nullptr, *inb = nullptr, *inq = nullptr, *inu = nullptr, *ilev = nullptr, *inlev = nullptr,
            *icons = nullptr, *incons = nullptr, *ictl = nullptr, *order = nullptr, *blkFirst = nullptr,
            *blkG = nullptr, *lcons = nullptr, *status = nullptr;
    int64_t *ybase = nullptr, *ystride = nullptr, *sbase = nullptr, *sstride = nullptr;
    double *grav = nullptr, *iparam = nullptr, *lst = nullptr, *time = nullptr;
    // staging
    int64_t upCap = 0, resCap = 0;  // bytes
    char* devUp = nullptr;
    char* devRes = nullptr;
    char* hostUp[2] = {nullptr, nullptr};
    char* hostRes[2] = {nullptr, nullptr};
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr, evTick[2] = {nullptr, nullptr}, evBegin[2] = {nullptr, nullptr};
    double gpuSeconds = 0;   // GPU time of the completed ticks
    double hostSeconds = 0;  // time inside sbg_server_tick ...
    double waitSeconds = 0;  // ... of which waiting for a tick in flight
    std::deque<TickRec> inflight;
    bool retryFailed = false;      // hand failed requests back for an FP64 rerun (mixed-precision tree lane)
    std::vector<int32_t> retry;    // their indices in reqs
    int64_t tick = 0;
    int64_t launches = 0;
    // requests
    std::mutex mu;
    std::vector<ServeReq> reqs;                    // by scheduler index
    std::unordered_map<int64_t, int32_t> byId;     // request id -> index
    int64_t nextId = 1, completed = 0, bodySteps = 0, peakResident = 0;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double clock() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    ~ServeLane() {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : bufs) cudaFree(p);
        for (int k = 0; k < 2; ++k) {
            if (hostUp[k]) cudaFreeHost(hostUp[k]);
            if (hostRes[k]) cudaFreeHost(hostRes[k]);
            if (evTick[k]) cudaEventDestroy(evTick[k]);
            if (evBegin[k]) cudaEventDestroy(evBegin[k]);
        }
        if (evFork) cudaEventDestroy(evFork);
        if (evJoin) cudaEventDestroy(evJoin);
        if (side) cudaStreamDestroy(side);
        if (stream) cudaStreamDestroy(stream);
    }
    template <class T_> int alloc(T_** out, int64_t count, const char* what) {
        void* p = nullptr;
        const size_t bytes = (size_t)std::max<int64_t>(count, 1) * sizeof(T_);
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return setError(SBG_ERR_NOMEM, std::string("server arena: cudaMalloc failed for ") + what + ": " +
                                               cudaGetErrorString(e));
        }
        bufs.push_back(p);
        devBytes += (int64_t)bytes;
        *out = static_cast<T_*>(p);
        return SBG_OK;
    }
};

namespace {

int cudaErr(cudaError_t e, const char* what) {
    return setError(SBG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define SBG_SCUDA(call, what)                                  \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cudaErr(e_, what);       \
    } while (0)

int64_t bytesPerUnit(int k, size_t rsz, bool fp64) {
    switch (k) {
    case kPoolRows: return kRowTables * 4 + kParamStride * (fp64 ? 8 : 8 + 4);
    case kPoolForces: return 4 + 2 * 8 + 2 * 4;
    case kPoolState: return 8 + 4 * (int64_t)rsz + (fp64 ? 0 : 4 * 8);
    case kPoolScratch: return (int64_t)rsz + (fp64 ? 0 : 8);  // mixed: + the FP64 mirror
    default: return 8;
    }
}

// Flatten a topology + request into its host image and footprint.
void buildImage(const sbg_topology_s& t, ServeReq& r, Footprint& fp) {
    const int nb = t.nb;
    const int rows = nb + 1;
    r.nb = nb;
    r.nq = t.nq;
    r.nu = t.nu;
    r.nlevels = t.nlevels;
    r.nf = (int)t.fkw.size();
    r.ncons = t.ncons;
    r.loops = t.ncons > 0;
    r.G = groupLanes(t);
    for (int k = 0; k < 3; ++k) r.grav[k] = t.gravity[k];
    int64_t recTotal = 0;
    const std::vector<int32_t> srec = paddedRecords(t, 3, &recTotal);
    r.rowsI.assign((size_t)kRowTables * rows, 0);
    auto at = [&](int table, int row) -> int32_t& { return r.rowsI[(size_t)table * rows + row]; };
    for (int i = 0; i < nb; ++i) {
        at(R_PARENT, i) = t.parent[i];
        at(R_INFO, i) = t.info[i];
        at(R_QOFF, i) = t.qoff[i];
        at(R_UOFF, i) = t.uoff[i];
        at(R_SREC, i) = srec[i];
        at(R_FBEG, i) = t.fbeg[i];  // request-relative: + force base at admission
        at(R_FCNT, i) = t.fcnt[i];
        at(R_LREC, i) = t.lslot[i] >= 0 ? (int32_t)(recTotal + (int64_t)t.lslot[i] * kSlotSize) : -1;
        at(R_LSLOT, i) = t.lslot[i];
        at(R_CBEG, i) = t.cbeg[i];  // request-relative: + row base at admission
        at(R_CCNT, i) = t.ccnt[i];
        at(R_KBEG, i) = t.kbeg[i];  // request-relative: + force base + nf at admission
        at(R_KCNT, i) = t.kcnt[i];
    }
    for (size_t i = 0; i < t.clist.size(); ++i) at(R_CLIST, (int)i) = t.clist[i];
    for (int L = 0; L <= t.nlevels; ++L) at(R_LEV, L) = t.levStart[L];
    r.par64 = t.par;
    r.fkw = t.fkw;
    r.fcoef = t.fcoef;
    r.fq0 = t.fq0;
    r.kpar = t.kpar;
    r.lcons = t.lcons;
    r.lst = t.lst;
    fp.units[kPoolRows] = rows;
    fp.units[kPoolForces] = r.nf + (int64_t)r.kpar.size();  // a contact takes kContactStride force units
    fp.units[kPoolState] = t.nq + t.nu;
    // level-parallel records: one row per body (loop closures: then the
    // slot rows, 2 per constraint), FP64 for loop closures
    r.recW = rowsRecordWidth(t, 3);
    if (r.loops) fp.units[kPoolLoopScratch] = (int64_t)(nb + 2 * t.ncons) * r.recW;
    else fp.units[kPoolScratch] = (int64_t)nb * r.recW;
}

// Upload staging of one tick: raw bytes plus the copy descriptors that move
// them to their device destinations (before the RK kernels), and the gather
// descriptors that collect finished states (after them).
struct Stager {
    ServeLane* s;
    char* host;
    int64_t cap, used = 0;
    std::vector<CopyDesc> pre, post;
    bool overflow = false;

    static int64_t pad16(int64_t b) { return (b + 15) & ~int64_t(15); }
    // Bytes of this tick's control arrays and descriptors for n resident
    // requests: order, block table and ictl entries with their descriptors,
    // and the three gather descriptors of a finishing request.
    static int64_t controlBytes(int64_t n) { return n * (4 + 8 + 16 + 4 * (int64_t)sizeof(CopyDesc)) + 4096; }
    // Room for `bytes` more data with `ndesc` more descriptors, keeping
    // `reserve` bytes for the control arrays.
    bool room(int64_t bytes, int ndesc, int64_t reserve) const {
        return used + pad16(bytes) + (int64_t)(pre.size() + post.size() + ndesc) * (int64_t)sizeof(CopyDesc) +
                   reserve <= cap;
    }
    // Stage `bytes` of host data for the device address dst.
    void put(const void* src, int64_t bytes, void* dst) {
        if (bytes <= 0) return;
        if (!room(bytes, 1, 0)) {
            overflow = true;
            return;
        }
        std::memcpy(host + used, src, (size_t)bytes);
        pre.push_back(CopyDesc{(uint64_t)(s->devUp + used), (uint64_t)dst, (uint32_t)(bytes / 4), 0});
        used += pad16(bytes);
    }
};

// Bytes the upload of one request takes in the staging buffer (and its
// descriptor count).
int64_t imageBytes(const ServeReq& r, size_t rsz, int* ndesc) {
    const int rows = r.nb + 1;
    int64_t b = 0;
    auto add = [&](int64_t x) { b += Stager::pad16(x); };
    for (int k = 0; k < kRowTables; ++k) add(rows * 4);
    add(r.par64.size() * 8);
    if (rsz == 4) add(r.par64.size() * 4);
    add(r.nf * 4);
    add(r.nf * 16);
    add(r.nf * 8);
    add((int64_t)r.kpar.size() * 8);
    add((int64_t)r.kpar.size() * 4);
    add((int64_t)r.y0.size() * 8);
    add(r.ncons * 2 * 4);
    add(r.ncons * 6 * 8);
    add(16 * 8);  // the slot's instance entries
    *ndesc = kRowTables + 2 + 5 + 2 + 1 + 2 + 16;
    return b;
}

// Stage the tables, state and instance entries of an admitted request.
void stageRequest(ServeLane* s, Stager& st, ServeReq& r, const SchedRequest& sr) {
    const int rows = r.nb + 1;
    const int64_t row0 = sr.off[kPoolRows], f0 = sr.off[kPoolForces], y0 = sr.off[kPoolState];
    const int slot = sr.slot;
    // row tables with the absolute fix-ups
    std::vector<int32_t> tab(r.rowsI);
    for (int i = 0; i < r.nb; ++i) {
        tab[(size_t)R_FBEG * rows + i] += (int32_t)f0;
        tab[(size_t)R_CBEG * rows + i] += (int32_t)row0;
        tab[(size_t)R_KBEG * rows + i] += (int32_t)(f0 + r.nf);
    }
    for (int k = 0; k < kRowTables; ++k) st.put(tab.data() + (size_t)k * rows, rows * 4, s->rowsI[k] + row0);
    st.put(r.par64.data(), (int64_t)r.par64.size() * 8, s->par64 + row0 * kParamStride);
    if (s->par32) {  // FP32 parameters of the mixed forms
        std::vector<float> p32(r.par64.begin(), r.par64.end());
        st.put(p32.data(), (int64_t)p32.size() * 4, s->par32 + row0 * kParamStride);
    }
    if (r.nf > 0) {
        std::vector<float> c32(r.fcoef.begin(), r.fcoef.end()), q32(r.fq0.begin(), r.fq0.end());
        st.put(r.fkw.data(), r.nf * 4, s->fkw + f0);
        st.put(r.fcoef.data(), r.nf * 8, s->fcoef64 + f0);
        st.put(r.fq0.data(), r.nf * 8, s->fq064 + f0);
        st.put(c32.data(), r.nf * 4, s->fcoef32 + f0);
        st.put(q32.data(), r.nf * 4, s->fq032 + f0);
    }
    if (!r.kpar.empty()) {  // contact values in the force pool after the forces
        const std::vector<float> k32(r.kpar.begin(), r.kpar.end());
        st.put(r.kpar.data(), (int64_t)r.kpar.size() * 8, s->fcoef64 + f0 + r.nf);
        st.put(k32.data(), (int64_t)k32.size() * 4, s->fcoef32 + f0 + r.nf);
    }
    st.put(r.y0.data(), (int64_t)r.y0.size() * 8, s->y + y0);
    if (r.ncons > 0) {
        st.put(r.lcons.data(), r.ncons * 2 * 4, s->lcons + (int64_t)slot * kMaxLoopCons * 2);
        st.put(r.lst.data(), r.ncons * 6 * 8, s->lst + (int64_t)slot * kMaxLoopCons * 6);
    }
    const int32_t ib = (int32_t)row0, nb = r.nb, nq = r.nq, nu = r.nu, nlev = r.nlevels,
                  ic = slot * kMaxLoopCons, nc = r.ncons, zero = 0;
    const int64_t yb = y0, one = 1, sb = r.loops ? sr.off[kPoolLoopScratch] : sr.off[kPoolScratch];
    // FP64 lanes: record-major rows of width recW (lane 0's serial loop work
    // revisits few records); trees: field-major, coalesced across the lanes
    // of a level (measured faster for them), sstride unused
    const int64_t sst = r.loops ? r.recW : 1;
    const double par[3] = {r.h, r.acc, r.ctol};
    st.put(&ib, 4, s->ibody + slot);
    st.put(&nb, 4, s->inb + slot);
    st.put(&nq, 4, s->inq + slot);
    st.put(&nu, 4, s->inu + slot);
    st.put(&ib, 4, s->ilev + slot);
    st.put(&nlev, 4, s->inlev + slot);
    st.put(&ic, 4, s->icons + slot);
    st.put(&nc, 4, s->incons + slot);
    st.put(&yb, 8, s->ybase + slot);
    st.put(&one, 8, s->ystride + slot);
    st.put(&sb, 8, s->sbase + slot);
    st.put(&sst, 8, s->sstride + slot);
    st.put(r.grav, 24, s->grav + 3 * (int64_t)slot);
    st.put(par, 24, s->iparam + 3 * (int64_t)slot);
    st.put(&r.t0, 8, s->time + slot);
    st.put(&zero, 4, s->status + slot);
}

// Copy finished requests out of the result buffer of a completed tick.
void harvest(ServeLane* s, const TickRec& tr) {
    const double now = s->clock();
    const char* base = s->hostRes[tr.parity];
    for (const auto& pr : tr.results) {
        ServeReq& r = s->reqs[s->byId[pr.first]];
        const char* p = base + pr.second;
        r.y.resize(r.nq + r.nu);
        std::memcpy(r.y.data(), p, r.y.size() * 8);
        std::memcpy(&r.t, p + r.y.size() * 8, 8);
        std::memcpy(&r.status, p + r.y.size() * 8 + 8, 4);
        if (r.status & (kStFp64 | kStWasFp64)) r.fp64Steps = 1;
        r.status &= ~(kStFp64 | kStWasFp64 | kStFp64LeftMask);
        if (s->retryFailed && (r.status & (SBG_INST_NONFINITE | SBG_INST_SINGULAR_D | SBG_INST_PROJECTION_FAILED))) {
            s->retry.push_back(s->byId[pr.first]);  // rerun from y0 in FP64; not done yet
            continue;
        }
        r.done = true;
        r.doneS = now;
        r.y0.clear();
        r.y0.shrink_to_fit();
        ++s->completed;
        s->bodySteps += (int64_t)r.nb * r.steps;
    }
}

// Wait for (block) or poll the oldest in-flight tick; harvest it when done.
int drainInflight(ServeLane* s, bool block, int32_t* ncompleted) {
    while (!s->inflight.empty()) {
        const TickRec& tr = s->inflight.front();
        const auto w0 = std::chrono::steady_clock::now();
        cudaError_t e = block ? cudaEventSynchronize(s->evTick[tr.parity]) : cudaEventQuery(s->evTick[tr.parity]);
        if (block) s->waitSeconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
        if (e == cudaErrorNotReady) {
            cudaGetLastError();
            return SBG_OK;
        }
        if (e != cudaSuccess) return cudaErr(e, "serving tick");
        float ms = 0;
        if (cudaEventElapsedTime(&ms, s->evBegin[tr.parity], s->evTick[tr.parity]) == cudaSuccess)
            s->gpuSeconds += 1e-3 * ms;
        else
            cudaGetLastError();
        const int64_t before = s->completed;
        harvest(s, tr);
        if (ncompleted) *ncompleted += (int32_t)(s->completed - before);
        s->inflight.pop_front();
        block = false;
    }
    return SBG_OK;
}

}  // namespace

namespace {

// One lane of the server: its own share of the budget (arena), slots,
// scheduler, stream and tick cadence.
int laneCreate(const sbg_server_config* cfg, int64_t budget, std::chrono::steady_clock::time_point t0,
               ServeLane** out) {
    auto* s = new (std::nothrow) ServeLane();
    if (!s) return setError(SBG_ERR_NOMEM, "out of host memory");
    auto bail = [&](int rc) { delete s; return rc; };
    s->t0 = t0;
    s->precision = cfg->precision;
    s->device = cfg->device;
    s->budget = budget;
    s->maxSlots = cfg->max_slots > 0 ? cfg->max_slots : 65536;
    s->chunk = cfg->chunk_steps > 0 ? std::min(cfg->chunk_steps, kCtlSteps) : 64;
    const bool fp64 = s->precision == SBG_PRECISION_FP64;
    s->rsz = fp64 ? 8 : 4;

    // Fixed part: slots, staging (device side), then the pools share the rest.
    const int64_t S = s->maxSlots;
    const int64_t slotBytes = S * (14 * 4 + 4 * 8 + (3 + 3 + 1) * 8 + kMaxLoopCons * (2 * 4 + 6 * 8)) + 2 * (S + 2) * 4;
    s->upCap = std::max<int64_t>(512 << 10, std::min<int64_t>(64 << 20, s->budget / 16));
    s->resCap = s->upCap;
    const int64_t fixed = slotBytes + s->upCap + s->resCap;
    if (fixed >= s->budget) return bail(setError(SBG_ERR_BUDGET, "device budget too small for the server's slots and staging"));
    double perRow = 0;
    for (int k = 0; k < kNumPools; ++k) perRow += kUnitsPerRow[k] * bytesPerUnit(k, s->rsz, fp64);
    const double rowsCap = double(s->budget - fixed) / perRow;
    for (int k = 0; k < kNumPools; ++k) s->cap[k] = std::max<int64_t>(kAlign[k], (int64_t)(rowsCap * kUnitsPerRow[k]));
    s->sched.configure(s->cap, kAlign, s->maxSlots, s->chunk);

    int rc = 0;
    const int64_t R = s->cap[kPoolRows];
    for (int k = 0; k < kRowTables; ++k)
        if ((rc = s->alloc(&s->rowsI[k], R, "body tables"))) return bail(rc);
    if ((rc = s->alloc(&s->par64, R * kParamStride, "parameters"))) return bail(rc);
    if (!fp64 && (rc = s->alloc(&s->par32, R * kParamStride, "parameters"))) return bail(rc);
    const int64_t F = s->cap[kPoolForces];
    if ((rc = s->alloc(&s->fkw, F, "forces")) || (rc = s->alloc(&s->fcoef64, F, "forces")) ||
        (rc = s->alloc(&s->fq064, F, "forces")) || (rc = s->alloc(&s->fcoef32, F, "forces")) ||
        (rc = s->alloc(&s->fq032, F, "forces")))
        return bail(rc);
    const int64_t Y = s->cap[kPoolState];
    if ((rc = s->alloc(&s->y, Y, "state"))) return bail(rc);
    if (fp64) {
        double* p = nullptr;
        if ((rc = s->alloc(&p, 4 * Y, "stage planes"))) return bail(rc);
        s->fbuf = s->fbufLoop = p;
    } else {
        float* p = nullptr;
        double* q = nullptr;
        if ((rc = s->alloc(&p, 4 * Y, "stage planes")) || (rc = s->alloc(&q, 4 * Y, "loop stage planes")))
            return bail(rc);
        s->fbuf = p;
        s->fbufLoop = q;
    }
    if (fp64) {
        double* p = nullptr;
        if ((rc = s->alloc(&p, s->cap[kPoolScratch], "scratch"))) return bail(rc);
        s->scratch = p;
    } else {
        float* p = nullptr;
        if ((rc = s->alloc(&p, s->cap[kPoolScratch], "scratch"))) return bail(rc);
        s->scratch = p;
        if ((rc = s->alloc(&s->scratch64, s->cap[kPoolScratch], "FP64 scratch mirror"))) return bail(rc);
    }
    if ((rc = s->alloc(&s->scratchLoop, s->cap[kPoolLoopScratch], "loop scratch"))) return bail(rc);
    int32_t** i32[] = {&s->ibody, &s->inb, &s->inq, &s->inu, &s->ilev, &s->inlev, &s->icons, &s->incons,
                       &s->ictl, &s->order, &s->status};
    for (auto p : i32)
        if ((rc = s->alloc(p, S, "slots"))) return bail(rc);
    if ((rc = s->alloc(&s->blkFirst, S + 2, "slots")) || (rc = s->alloc(&s->blkG, S + 2, "slots")) ||
        (rc = s->alloc(&s->lcons, S * kMaxLoopCons * 2, "slots")) ||
        (rc = s->alloc(&s->lst, S * kMaxLoopCons * 6, "slots")) || (rc = s->alloc(&s->ybase, S, "slots")) ||
        (rc = s->alloc(&s->ystride, S, "slots")) || (rc = s->alloc(&s->sbase, S, "slots")) ||
        (rc = s->alloc(&s->sstride, S, "slots")) || (rc = s->alloc(&s->grav, 3 * S, "slots")) ||
        (rc = s->alloc(&s->iparam, 3 * S, "slots")) || (rc = s->alloc(&s->time, S, "slots")))
        return bail(rc);
    if ((rc = s->alloc(&s->devUp, s->upCap, "staging")) || (rc = s->alloc(&s->devRes, s->resCap, "staging")))
        return bail(rc);
    for (int k = 0; k < 2; ++k) {
        cudaError_t e = cudaMallocHost(&s->hostUp[k], (size_t)s->upCap);
        if (e == cudaSuccess) e = cudaMallocHost(&s->hostRes[k], (size_t)s->resCap);
        if (e == cudaSuccess) e = cudaEventCreate(&s->evTick[k]);
        if (e == cudaSuccess) e = cudaEventCreate(&s->evBegin[k]);
        if (e != cudaSuccess) return bail(cudaErr(e, "pinned staging"));
    }
    {
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->evFork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->evJoin, cudaEventDisableTiming);
        if (e != cudaSuccess) return bail(cudaErr(e, "streams"));
    }
    DevTables& T = s->T;
    T.parent = s->rowsI[R_PARENT];
    T.info = s->rowsI[R_INFO];
    T.qoff = s->rowsI[R_QOFF];
    T.uoff = s->rowsI[R_UOFF];
    T.srec = s->rowsI[R_SREC];
    T.fbeg = s->rowsI[R_FBEG];
    T.fcnt = s->rowsI[R_FCNT];
    T.lrec = s->rowsI[R_LREC];
    T.lslot = s->rowsI[R_LSLOT];
    T.cbeg = s->rowsI[R_CBEG];
    T.ccnt = s->rowsI[R_CCNT];
    T.clist = s->rowsI[R_CLIST];
    T.levStart = s->rowsI[R_LEV];
    T.par64 = s->par64;
    T.par32 = s->par32;
    T.fkind_which = s->fkw;
    T.fcoef64 = s->fcoef64;
    T.fq064 = s->fq064;
    T.fcoef32 = s->fcoef32;
    T.fq032 = s->fq032;
    T.kbeg = s->rowsI[R_KBEG];
    T.kcnt = s->rowsI[R_KCNT];
    T.kpar64 = s->fcoef64;
    T.kpar32 = s->fcoef32;
    T.ibody = s->ibody;
    T.inb = s->inb;
    T.inq = s->inq;
    T.inu = s->inu;
    T.ybase = s->ybase;
    T.ystride = s->ystride;
    T.sbase = s->sbase;
    T.sstride = s->sstride;
    T.grav = s->grav;
    T.order = s->order;
    T.ninst = (int32_t)S;
    T.ilev = s->ilev;
    T.inlev = s->inlev;
    T.blkFirst = s->blkFirst;
    T.blkG = s->blkG;
    T.lcons = s->lcons;
    T.lst = s->lst;
    T.icons = s->icons;
    T.incons = s->incons;
    T.ictl = s->ictl;
    T.iparam = s->iparam;
    T.scratch64 = s->scratch64;
    *out = s;
    return SBG_OK;
}

// Queue a request whose image, footprint and cost are set (the caller holds
// the lane's mutex).
int laneEnqueue(ServeLane* s, ServeReq&& r) {
    if (!s->sched.fitsEver(r.fp))
        return setError(SBG_ERR_BUDGET, "request needs more device memory than the server's budget provides");
    int nd = 0;
    if (imageBytes(r, s->rsz, &nd) + (int64_t)nd * (int64_t)sizeof(CopyDesc) + Stager::controlBytes(1) > s->upCap / 2)
        return setError(SBG_ERR_BUDGET, "request's tables exceed the server's upload staging");
    if ((int64_t)(r.nq + r.nu) * 8 + 16 > s->resCap)
        return setError(SBG_ERR_BUDGET, "request's state exceeds the server's result staging");
    const int32_t chunk =
        (int32_t)std::max(1.0, std::min(16.0 * s->chunk, std::floor(s->chunk * kRefCost / std::max(r.cost, 1e-9))));
    r.sched = s->sched.submit(r.id, r.fp, (int32_t)r.steps, chunk);
    s->byId[r.id] = r.sched;
    s->reqs.push_back(std::move(r));
    return SBG_OK;
}

// Queue a request on a lane (the caller holds the lane's mutex).
int laneSubmit(ServeLane* s, int64_t rid, sbg_topology topo, const double* y0, double t0, double h, int32_t nsteps,
               const sbg_integ_opts* opts) {
    ServeReq r;
    Footprint fp;
    buildImage(*topo, r, fp);
    r.y0.assign(y0, y0 + topo->nq + topo->nu);
    r.t0 = t0;
    r.h = h;
    r.steps = nsteps;
    double acc = 1e-3, ctol = -1;
    if (opts) {
        if (opts->accuracy > 0) acc = opts->accuracy;
        if (opts->constraint_tolerance > 0) ctol = opts->constraint_tolerance;
        r.pes = opts->project_every_step != 0;
    }
    r.acc = acc;
    r.ctol = ctol > 0 ? ctol : acc / 10;
    r.id = rid;
    r.submitS = s->clock();
    r.cost = stepCost(*topo, r.loops, r.G);
    r.fp = fp;
    return laneEnqueue(s, std::move(r));
}

int laneIssue(ServeLane* s);

// One scheduling round of a lane. Results of finished ticks are collected;
// a new tick is prepared only while at most one is in flight (its staging
// buffers alternate by parity): with `block`, by waiting for the older one,
// otherwise by returning at once (*issued = false).
int laneTick(ServeLane* s, bool block, int32_t* ncompleted, bool* issued) {
    *issued = false;
    if (int rc = drainInflight(s, false, ncompleted)) return rc;
    if (s->inflight.size() >= 2) {
        if (!block) return SBG_OK;
        if (int rc = drainInflight(s, true, ncompleted)) return rc;
    }
    if (s->inflight.size() >= 2) return setError(SBG_ERR_STATE, "serving ticks did not complete");
    const int64_t tick0 = s->tick;
    const int rc = laneIssue(s);
    *issued = s->tick != tick0;
    return rc;
}

int laneIssue(ServeLane* s) {
    const int parity = (int)(s->tick & 1);
    Stager st{s, s->hostUp[parity], s->upCap};
    const double now = s->clock();
    // 2. admission, keeping room for the control arrays of every resident
    //    request (the ones admitted so far included)
    std::vector<int32_t> admitted = s->sched.admit(s->tick, [&](int32_t i) {
        int nd = 0;
        const int64_t b = imageBytes(s->reqs[i], s->rsz, &nd);
        if (!st.room(b, nd, Stager::controlBytes((int64_t)s->sched.resident() + 1))) return false;
        stageRequest(s, st, s->reqs[i], s->sched.req(i));
        return true;
    });
    for (int32_t i : admitted) s->reqs[i].admitS = now;
    // 3. plan: every resident request runs one chunk; finishing ones need
    //    room in the result buffer
    int64_t resUsed = 0;
    std::vector<std::pair<int32_t, int64_t>> finishing;  // (request index, result offset)
    std::vector<PlannedChunk> plan = s->sched.plan(s->tick, [&](int32_t i) {
        const int64_t need = Stager::pad16((int64_t)(s->reqs[i].nq + s->reqs[i].nu) * 8 + 16);
        if (resUsed + need > s->resCap) return false;
        finishing.emplace_back(i, resUsed);
        resUsed += need;
        return true;
    });
    if (plan.empty() && admitted.empty()) return SBG_OK;
    s->peakResident = std::max<int64_t>(s->peakResident, (int64_t)plan.size());
    // 4. control arrays. Two level-parallel segments, each sorted by lanes
    //    per request (widest first) and cut into 128-thread blocks of equal
    //    lanes: loop-closure requests (FP64, blocks [0, nLoopBlocks)) and
    //    the other trees (the server's precision, the blocks after them).
    std::vector<int32_t> loopIdx, grpIdx;
    for (const PlannedChunk& c : plan) (s->reqs[c.req].loops ? loopIdx : grpIdx).push_back((int32_t)(&c - plan.data()));
    auto byLanes = [&](int32_t a, int32_t b) { return s->reqs[plan[a].req].G > s->reqs[plan[b].req].G; };
    std::stable_sort(loopIdx.begin(), loopIdx.end(), byLanes);
    std::stable_sort(grpIdx.begin(), grpIdx.end(), byLanes);
    std::vector<int32_t> order, blkFirst, blkG;
    order.reserve(plan.size());
    auto segment = [&](const std::vector<int32_t>& idx) {
        const int32_t pos0 = (int32_t)order.size();
        for (size_t p = 0; p < idx.size();) {
            const int G = s->reqs[plan[idx[p]].req].G;
            size_t q = p;
            while (q < idx.size() && (int)(q - p) < 128 / G && s->reqs[plan[idx[q]].req].G == G) ++q;
            blkFirst.push_back(pos0 + (int32_t)p);
            blkG.push_back(G);
            p = q;
        }
        for (int32_t k : idx) order.push_back(s->sched.req(plan[k].req).slot);
    };
    segment(loopIdx);
    const int nLoopBlocks = (int)blkFirst.size();
    segment(grpIdx);
    const int nGroupBlocks = (int)blkFirst.size() - nLoopBlocks;
    blkFirst.push_back((int32_t)order.size());
    blkG.push_back(0);
    if (!order.empty()) st.put(order.data(), (int64_t)order.size() * 4, s->order);
    st.put(blkFirst.data(), (int64_t)blkFirst.size() * 4, s->blkFirst);
    st.put(blkG.data(), (int64_t)blkG.size() * 4, s->blkG);
    for (const PlannedChunk& c : plan) {
        const ServeReq& r = s->reqs[c.req];
        const int32_t w = c.steps | (c.first ? kCtlInit : 0) | (r.pes ? kCtlProjectEveryStep : 0);
        st.put(&w, 4, s->ictl + s->sched.req(c.req).slot);
    }
    // gathers of the finishing requests: y, then t and the status word
    TickRec tr;
    tr.parity = parity;
    for (const auto& f : finishing) {
        const ServeReq& r = s->reqs[f.first];
        const SchedRequest& sr = s->sched.req(f.first);
        const int64_t ny = r.nq + r.nu;
        char* dst = s->devRes + f.second;
        st.post.push_back(CopyDesc{(uint64_t)(s->y + sr.off[kPoolState]), (uint64_t)dst, (uint32_t)(ny * 2), 0});
        st.post.push_back(CopyDesc{(uint64_t)(s->time + sr.slot), (uint64_t)(dst + ny * 8), 2, 0});
        st.post.push_back(CopyDesc{(uint64_t)(s->status + sr.slot), (uint64_t)(dst + ny * 8 + 8), 1, 0});
        tr.results.emplace_back(r.id, f.second);
    }
    // descriptor lists at the end of the staged bytes
    const int64_t preOff = st.used;
    const int64_t postOff = preOff + (int64_t)st.pre.size() * (int64_t)sizeof(CopyDesc);
    const int64_t upBytes = postOff + (int64_t)st.post.size() * (int64_t)sizeof(CopyDesc);
    if (st.overflow || upBytes > s->upCap)
        return setError(SBG_ERR_STATE, "serving tick does not fit the upload staging (too many resident requests)");
    std::memcpy(st.host + preOff, st.pre.data(), st.pre.size() * sizeof(CopyDesc));
    std::memcpy(st.host + postOff, st.post.data(), st.post.size() * sizeof(CopyDesc));
    // 5. enqueue the tick
    cudaStream_t m = s->stream;
    SBG_SCUDA(cudaEventRecord(s->evBegin[parity], m), "tick event");
    SBG_SCUDA(cudaMemcpyAsync(s->devUp, st.host, (size_t)upBytes, cudaMemcpyHostToDevice, m), "tick upload");
    SBG_SCUDA(launchCopies(reinterpret_cast<const CopyDesc*>(s->devUp + preOff), (int)st.pre.size(), m), "tick scatter");
    ++s->launches;
    if (!plan.empty()) {
        LaunchPlan P{};
        P.nm = 3;
        P.variant = 1;
        P.nGroupBlocks = nGroupBlocks;
        P.groupFirst = nLoopBlocks;
        P.nLoopGroupBlocks = nLoopBlocks;
        P.loopGroupFirst = 0;
        KArgs a{};
        a.T = &s->T;
        a.P = &P;
        a.ystate = s->y;
        a.time = s->time;
        a.fbuf = s->fbuf;
        a.fbufLoop = s->fbufLoop;
        a.fplane = s->cap[kPoolState];
        a.scratch = s->scratch;
        a.scratchLoop = s->scratchLoop;
        a.status = s->status;
        a.h = 0;
        a.step = StepCtl{0, 0, 0.0, 0, 0};  // per instance from ictl/iparam
        a.accuracy = 1e-3;
        a.consTol = 1e-4;
        const bool both = nLoopBlocks > 0 && nGroupBlocks > 0;
        cudaStream_t gs = both ? s->side : m;
        if (both) {
            SBG_SCUDA(cudaEventRecord(s->evFork, m), "fork");
            SBG_SCUDA(cudaStreamWaitEvent(s->side, s->evFork, 0), "fork");
        }
        if (nGroupBlocks > 0) {
            if (s->precision == SBG_PRECISION_FP64) rk64Group(a, gs);
            else rk32Group(a, s->precision == SBG_PRECISION_MIXED, gs);
            ++s->launches;
        }
        if (nLoopBlocks > 0) {
            rkLoopGroup(a, m);
            ++s->launches;
        }
        if (both) {
            SBG_SCUDA(cudaEventRecord(s->evJoin, s->side), "join");
            SBG_SCUDA(cudaStreamWaitEvent(m, s->evJoin, 0), "join");
        }
        SBG_SCUDA(cudaGetLastError(), "serving RK-Merson launch");
    }
    if (!st.post.empty()) {
        SBG_SCUDA(launchCopies(reinterpret_cast<const CopyDesc*>(s->devUp + postOff), (int)st.post.size(), m),
                  "tick gather");
        ++s->launches;
        SBG_SCUDA(cudaMemcpyAsync(s->hostRes[parity], s->devRes, (size_t)resUsed, cudaMemcpyDeviceToHost, m),
                  "tick download");
    }
    SBG_SCUDA(cudaEventRecord(s->evTick[parity], m), "tick event");
    // Finished requests give their memory and slot back now: whatever is
    // uploaded into them later is ordered after this tick on the stream.
    for (const auto& f : finishing) s->sched.retire(f.first);
    s->inflight.push_back(std::move(tr));
    ++s->tick;
    return SBG_OK;
}

bool laneIdle(const ServeLane* s) { return s->sched.queued() == 0 && s->sched.resident() == 0; }

}  // namespace

// The server: lanes with independent tick cadences, so that requests of very
// different cost per step do not wait on each other (a tick lasts at least
// one step of its costliest request). Lane 0 runs the trees without loop
// closures (level-parallel driver, the server's precision); lanes 1 and 2
// run in FP64 the trees with Ball loop closures (multiplier solve and
// projections) and the reruns of failed mixed-precision requests, split by
// estimated cost per step at kSplitCost. The budget and the slots are split
// in proportion to the lanes' expected share of the arena.
constexpr int kLanes = 3;
constexpr double kLaneShare[kLanes] = {0.65, 0.20, 0.15};
constexpr double kSplitCost = 200.0;  // stepCost units: about the median loop-closure request
int fp64Lane(double cost) { return cost <= kSplitCost ? 1 : 2; }

struct sbg_server_s {
    ServeLane* lane[kLanes] = {nullptr, nullptr, nullptr};
    std::mutex mu;
    int64_t nextId = 1;
    std::unordered_map<int64_t, int> laneOf;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double hostSeconds = 0;  // inside sbg_server_tick ...
    double pollSeconds = 0;  // ... of which waiting for a lane to free up
    ~sbg_server_s() {
        for (ServeLane* L : lane) delete L;
    }
    double clock() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

// Requests whose mixed-precision run failed (non-finite, singular D, failed
// projection) start again from their initial state in the FP64 lane, as the
// reference's integrator restores the state and reports StepFailed
// (AbstractIntegratorRep.cpp:426-431); their latency counts from the first
// submission. Every lane's mutex is held by the caller.
int moveRetries(sbg_server_s* s) {
    ServeLane* A = s->lane[0];
    for (int32_t i : A->retry) {
        ServeReq& a = A->reqs[i];
        ServeReq r;
        r.id = a.id;
        r.loops = true;  // the FP64 lane's level-parallel segment (no constraints: no loop work)
        r.G = a.G;
        r.nb = a.nb; r.nq = a.nq; r.nu = a.nu; r.nlevels = a.nlevels; r.nf = a.nf; r.ncons = a.ncons;
        r.recW = a.recW;
        r.t0 = a.t0; r.h = a.h; r.acc = a.acc; r.ctol = a.ctol; r.pes = a.pes;
        for (int k = 0; k < 3; ++k) r.grav[k] = a.grav[k];
        r.rowsI = a.rowsI; r.par64 = a.par64; r.fkw = a.fkw; r.fcoef = a.fcoef; r.fq0 = a.fq0; r.kpar = a.kpar;
        r.lcons = a.lcons; r.lst = a.lst; r.y0 = a.y0;
        r.steps = a.steps;
        r.submitS = a.submitS;
        r.attempts = 2;
        r.fp = a.fp;
        r.fp.units[kPoolLoopScratch] = a.fp.units[kPoolScratch];  // same records, in FP64
        r.fp.units[kPoolScratch] = 0;
        r.cost = a.cost * kLoopDriverWeight;
        const int li = fp64Lane(r.cost);
        if (int rc = laneEnqueue(s->lane[li], std::move(r))) return rc;
        s->laneOf[a.id] = li;
        a.y0.clear();
        a.y0.shrink_to_fit();
    }
    A->retry.clear();
    return SBG_OK;
}

extern "C" {

int sbg_server_create(const sbg_server_config* cfg, sbg_server* out) {
    if (!cfg || !out) return setError(SBG_ERR_INVALID, "null argument");
    if (cfg->precision != SBG_PRECISION_FP64 && cfg->precision != SBG_PRECISION_MIXED &&
        cfg->precision != SBG_PRECISION_MIXED_FAST)
        return setError(SBG_ERR_INVALID, "unknown precision");
    if (cfg->device_budget_bytes <= 0) return setError(SBG_ERR_INVALID, "the server needs a positive device budget");
    if (cfg->max_slots < 0 || cfg->chunk_steps < 0) return setError(SBG_ERR_INVALID, "negative slot count or chunk");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return setError(SBG_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (cfg->device < 0 || cfg->device >= ndev) return setError(SBG_ERR_INVALID, "bad device ordinal");
    SBG_SCUDA(cudaSetDevice(cfg->device), "cudaSetDevice");
    auto* s = new (std::nothrow) sbg_server_s();
    if (!s) return setError(SBG_ERR_NOMEM, "out of host memory");
    const int32_t slots = cfg->max_slots > 0 ? cfg->max_slots : 65536;
    if (slots < kLanes) {
        delete s;
        return setError(SBG_ERR_INVALID, "the server needs at least " + std::to_string(kLanes) + " slots (one per lane)");
    }
    int32_t left = slots;
    int64_t budgetLeft = cfg->device_budget_bytes;
    for (int li = kLanes - 1; li >= 0; --li) {  // lane 0 takes what the others leave
        sbg_server_config c = *cfg;
        c.max_slots = li == 0 ? left : std::max(1, std::min(left - li, (int32_t)std::lround(slots * kLaneShare[li])));
        const int64_t budget = li == 0 ? budgetLeft : (int64_t)(cfg->device_budget_bytes * kLaneShare[li]);
        left -= c.max_slots;
        budgetLeft -= budget;
        if (int rc = laneCreate(&c, budget, s->t0, &s->lane[li])) {
            delete s;
            return rc;
        }
    }
    s->lane[0]->retryFailed = cfg->precision != SBG_PRECISION_FP64;
    *out = s;
    return SBG_OK;
}

int sbg_server_destroy(sbg_server s) {
    delete s;
    return SBG_OK;
}

int sbg_server_submit(sbg_server s, sbg_topology topo, const double* y0, double t0, double h, int32_t nsteps,
                      const sbg_integ_opts* opts, int64_t* id) {
    if (!s || !topo || !y0 || !id) return setError(SBG_ERR_INVALID, "null argument");
    if (!(h > 0) || !std::isfinite(h)) return setError(SBG_ERR_INVALID, "step size must be positive");
    if (nsteps < 0 || nsteps > kCtlSteps) return setError(SBG_ERR_INVALID, "step count out of range");
    if (topo->ncons > kMaxLoopCons)
        return setError(SBG_ERR_UNSUPPORTED, "at most " + std::to_string(kMaxLoopCons) + " Ball loop closures per system");
    std::lock_guard<std::mutex> lock(s->mu);
    const bool loops = topo->ncons > 0;
    const int li = loops ? fp64Lane(stepCost(*topo, true, groupLanes(*topo))) : 0;
    ServeLane* L = s->lane[li];
    std::lock_guard<std::mutex> lk(L->mu);
    const int64_t rid = s->nextId;
    if (int rc = laneSubmit(L, rid, topo, y0, t0, h, nsteps, opts)) return rc;
    ++s->nextId;
    s->laneOf[rid] = li;
    *id = rid;
    return SBG_OK;
}

int sbg_server_tick(sbg_server s, int32_t* ncompleted) {
    if (!s) return setError(SBG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lock(s->mu);
    if (ncompleted) *ncompleted = 0;
    SBG_SCUDA(cudaSetDevice(s->lane[0]->device), "cudaSetDevice");
    const auto h0 = std::chrono::steady_clock::now();
    // Each lane issues its next tick when it can; if neither can (both have
    // two ticks in flight), wait for whichever finishes first.
    for (int round = 0;; ++round) {
        bool any = false, work = false;
        for (ServeLane* L : s->lane) {
            std::lock_guard<std::mutex> lk(L->mu);
            int32_t n = 0;
            bool issued = false;
            if (int rc = laneTick(L, false, &n, &issued)) return rc;
            if (ncompleted) *ncompleted += n;
            any |= issued || n > 0;
            work |= !L->inflight.empty();  // waiting for a tick in flight can free a lane
        }
        {
            std::lock_guard<std::mutex> l0(s->lane[0]->mu);
            std::lock_guard<std::mutex> l1(s->lane[1]->mu);
            std::lock_guard<std::mutex> l2(s->lane[2]->mu);
            any |= !s->lane[0]->retry.empty();
            if (int rc = moveRetries(s)) return rc;
        }
        if (any || !work) break;
        const auto w0 = std::chrono::steady_clock::now();
        std::this_thread::sleep_for(std::chrono::microseconds(round < 100 ? 20 : 200));
        s->pollSeconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    }
    s->hostSeconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - h0).count();
    return SBG_OK;
}

int sbg_server_drain(sbg_server s) {
    if (!s) return setError(SBG_ERR_INVALID, "null server");
    for (ServeLane* L : s->lane) {  // the tree lane first: its failures join the FP64 lanes
        for (;;) {
            std::lock_guard<std::mutex> lock(s->mu);
            std::lock_guard<std::mutex> lk(L->mu);
            if (laneIdle(L)) {
                if (int rc = drainInflight(L, true, nullptr)) return rc;
                if (L->inflight.empty()) break;
            }
            int32_t n = 0;
            bool issued = false;
            if (int rc = laneTick(L, true, &n, &issued)) return rc;
            if (!issued && L->inflight.empty() && !laneIdle(L))
                return setError(SBG_ERR_STATE, "serving made no progress: a queued request cannot be admitted");
        }
        std::lock_guard<std::mutex> lock(s->mu);
        std::lock_guard<std::mutex> l0(s->lane[0]->mu);
        std::lock_guard<std::mutex> l1(s->lane[1]->mu);
        std::lock_guard<std::mutex> l2(s->lane[2]->mu);
        if (int rc = moveRetries(s)) return rc;
    }
    return SBG_OK;
}

int sbg_server_result(sbg_server s, int64_t id, double* y, sbg_request_info* info) {
    if (!s) return setError(SBG_ERR_INVALID, "null server");
    std::lock_guard<std::mutex> lock0(s->mu);
    auto li = s->laneOf.find(id);
    if (li == s->laneOf.end()) return setError(SBG_ERR_INVALID, "unknown request id");
    ServeLane* L = s->lane[li->second];
    std::lock_guard<std::mutex> lock(L->mu);
    auto it = L->byId.find(id);
    if (it == L->byId.end()) return setError(SBG_ERR_INVALID, "unknown request id");
    const ServeReq& r = L->reqs[it->second];
    if (info) {
        info->done = r.done ? 1 : 0;
        info->status = r.status;
        info->nbodies = r.nb;
        info->nsteps = (int32_t)r.steps;
        info->t = r.t;
        info->submit_s = r.submitS;
        info->admit_s = r.admitS;
        info->done_s = r.doneS;
        info->attempts = r.attempts;
        info->fp64_steps = r.fp64Steps;
    }
    if (!r.done) return info ? SBG_OK : setError(SBG_ERR_STATE, "request not finished");
    if (y) std::memcpy(y, r.y.data(), r.y.size() * 8);
    return SBG_OK;
}

int sbg_server_get_stats(sbg_server s, sbg_server_stats* out) {
    if (!s || !out) return setError(SBG_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lock0(s->mu);
    std::memset(out, 0, sizeof *out);
    double wait = 0;
    out->submitted = s->nextId - 1;  // FP64 reruns are not new submissions
    for (ServeLane* L : s->lane) {
        std::lock_guard<std::mutex> lock(L->mu);
        out->completed += L->completed;
        out->queued += (int64_t)L->sched.queued();
        out->resident += (int64_t)L->sched.resident();
        out->peak_resident += L->peakResident;
        out->ticks += L->tick;
        out->launches += L->launches;
        out->body_steps += L->bodySteps;
        out->device_bytes += L->devBytes;
        out->max_slots += L->maxSlots;
        out->chunk_steps = L->chunk;
        out->gpu_seconds += L->gpuSeconds;
        wait += L->waitSeconds;
        for (int k = 0; k < kNumPools; ++k) {
            out->pool_capacity[k] += L->sched.pool(k).capacity();
            out->pool_in_use[k] += L->sched.pool(k).used();
        }
    }
    out->host_seconds = s->hostSeconds - wait - s->pollSeconds;
    return SBG_OK;
}

int sbg_server_get_lane_stats(sbg_server s, int32_t lane, sbg_server_stats* out) {
    if (!s || !out || lane < 0 || lane >= kLanes) return setError(SBG_ERR_INVALID, "bad argument");
    std::lock_guard<std::mutex> lock0(s->mu);
    ServeLane* L = s->lane[lane];
    std::lock_guard<std::mutex> lock(L->mu);
    std::memset(out, 0, sizeof *out);
    out->submitted = (int64_t)L->reqs.size();
    out->completed = L->completed;
    out->queued = (int64_t)L->sched.queued();
    out->resident = (int64_t)L->sched.resident();
    out->peak_resident = L->peakResident;
    out->ticks = L->tick;
    out->launches = L->launches;
    out->body_steps = L->bodySteps;
    out->device_bytes = L->devBytes;
    out->max_slots = L->maxSlots;
    out->chunk_steps = L->chunk;
    out->gpu_seconds = L->gpuSeconds;
    out->host_seconds = 0;
    for (int k = 0; k < kNumPools; ++k) {
        out->pool_capacity[k] = L->sched.pool(k).capacity();
        out->pool_in_use[k] = L->sched.pool(k).used();
    }
    return SBG_OK;
}

double sbg_server_clock(sbg_server s) { return s ? s->clock() : 0.0; }

// The scheduler without a device: requests arrive at given ticks; every
// tick admits, plans and retires exactly as sbg_server_tick does.
int sbg_serve_simulate(int32_t n, const int64_t* units, const int32_t* horizons, const int64_t* arrivalTick,
                       const int64_t* capacity, int32_t maxSlots, int32_t chunk, int64_t* admitTick,
                       int64_t* doneTick, int64_t* peakResident) {
    if (n < 0 || (n > 0 && (!units || !horizons || !arrivalTick || !admitTick || !doneTick)) || !capacity ||
        maxSlots <= 0 || chunk <= 0)
        return setError(SBG_ERR_INVALID, "bad simulation arguments");
    Scheduler sc;
    sc.configure(capacity, kAlign, maxSlots, chunk);
    std::vector<int32_t> idx(n, -1);
    for (int i = 0; i < n; ++i) {
        Footprint fp;
        for (int k = 0; k < kNumPools; ++k) fp.units[k] = units[(int64_t)i * kNumPools + k];
        if (!sc.fitsEver(fp)) return setError(SBG_ERR_BUDGET, "request " + std::to_string(i) + " never fits");
        if (horizons[i] < 0) return setError(SBG_ERR_INVALID, "negative horizon");
    }
    int next = 0, done = 0;
    int64_t peak = 0;
    for (int64_t tick = 0; done < n; ++tick) {
        while (next < n && arrivalTick[next] <= tick) {
            Footprint fp;
            for (int k = 0; k < kNumPools; ++k) fp.units[k] = units[(int64_t)next * kNumPools + k];
            idx[next] = sc.submit(next, fp, horizons[next]);
            ++next;
        }
        for (int32_t i : sc.admit(tick)) admitTick[sc.req(i).id] = tick;
        const std::vector<PlannedChunk> p = sc.plan(tick);
        peak = std::max<int64_t>(peak, (int64_t)p.size());
        for (const PlannedChunk& c : p)
            if (c.last) {
                doneTick[sc.req(c.req).id] = tick;
                sc.retire(c.req);
                ++done;
            }
        if (tick > (int64_t)1 << 40) return setError(SBG_ERR_STATE, "simulation did not finish");
    }
    if (peakResident) *peakResident = peak;
    return SBG_OK;
}

}  // extern "C"
