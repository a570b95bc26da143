// capi.cpp -- host runtime behind the C ABI of include/simbody_gb300.h:
// topology flattening, batch memory management and kernel dispatch.
#include "../../include/simbody_gb300.h"
#include "engine.h"
#include "kernels.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

using namespace sbg;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
int cudaFail(cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return SBG_ERR_CUDA;
}
#define SBG_CUDA(call, what)                                   \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return cudaFail(e_, what);      \
    } while (0)

// q and u slots per mobilizer (sbg_mobilizer order). Ball and Free keep 4
// and 7 q slots in Euler-angle mode too, the last one unused, as Simbody's
// State does (RigidBodyNodeSpec_Ball.h:393-395).
const int kNQ[SBG_NUM_MOBILIZERS] = {1, 1, 2, 4, 7, 3, 3, 2, 3, 6, 0, 1};
const int kNU[SBG_NUM_MOBILIZERS] = {1, 1, 2, 3, 6, 3, 3, 2, 3, 6, 0, 1};

// Host buffers the caller allocated page-locked (cudaMallocHost,
// cudaHostRegister, a pinned torch tensor) are copied to and from directly;
// pageable ones go through the batch's pinned staging buffer.
bool isPinned(const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

bool isIdentityR(const double* X) {
    return X[0] == 1 && X[1] == 0 && X[2] == 0 && X[3] == 0 && X[4] == 1 && X[5] == 0 && X[6] == 0 && X[7] == 0 &&
           X[8] == 1;
}

}  // namespace

#include "topology_internal.h"

namespace sbg {
int setError(int code, const std::string& msg) {
    g_err = msg;
    return code;
}
}  // namespace sbg

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct sbg_batch_s {
    int precision = 0, device = 0;
    int64_t budget = 0;
    int ninst = 0;
    int nm = 3;
    bool tiled = false;
    int variant = 0;  // kernel variant: 0 = not tuned yet, else 1, 4, 7 or 8 (see LaunchPlan)
    bool stagedOk = false;  // variant 8 applies: one shared chain topology without Free bodies
    cudaStream_t stream = nullptr;
    std::vector<int32_t> instTopo;
    std::vector<int64_t> hostYOff, hostUOff;  // packed host offsets (n+1)
    std::vector<int64_t> hostBOff;            // bodies before each instance (n+1)
    int64_t nyTotal = 0, nuTotal = 0, colElems = 0;
    std::vector<DevBuf> bufs;
    int64_t devBytes = 0;
    DevTables T{};
    // device pointers
    double* y = nullptr;       // state columns
    double* ydot = nullptr;    // derivative columns
    double* fcol = nullptr;    // M^-1 input columns
    double* time = nullptr;
    int32_t* status = nullptr;
    int64_t* dHostYOff = nullptr;
    int64_t* dHostUOff = nullptr;
    int64_t* dHostQOff = nullptr;  // qdotdot packing: nq values per instance
    double* staging = nullptr;  // packed device staging (nyTotal)
    void* scratch = nullptr;
    void* fbuf = nullptr;       // RK stage derivatives, 4 planes
    void* scratchLoop = nullptr;  // FP64 scratch of the loop-closure segment
    void* fbufLoop = nullptr;     // FP64 stage derivatives of that segment (fbuf itself in FP64 batches)
    int nLoop = 0;                // order positions [nChain, nChain + nLoop)
    int64_t scratchElems = 0;
    double* hostPinned = nullptr;  // pinned host staging (nyTotal)
    bool stateSet = false;
    bool integrating = false;  // an integration has run since the state was last set: it can be continued
    bool realized = false;     // ydot holds the realize of the current state (qdotdot can be formed)
    int64_t launches = 0;
    // mapping
    int nChain = 0;                       // order positions of the chain segment
    std::vector<int32_t> groupWidthKey;   // widest level of each group-segment instance
    int groupShift = -1;                  // G = pow2ceil(width) >> shift, clamped to [2, 32]
    int nGroupBlocks = 0;
    int32_t* dBlkFirst = nullptr;
    int32_t* dBlkG = nullptr;
    cudaStream_t stream2 = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    bool orderIdentity = false;         // launch order = instance order (a one-topology chain batch)
    // pipelined host realize: pipe[0] (= stream) uploads the chunks in order,
    // pipe[1..3] compute them, pipe[4] downloads them in order; per chunk an
    // event when its upload and when its gather is done
    cudaStream_t pipe[5] = {};
    cudaEvent_t pipeEv[2][16] = {};
    cudaEvent_t pipeStart = nullptr, pipeEnd = nullptr;
    cudaEvent_t evT0 = nullptr, evT1 = nullptr;
    bool tuned = false;
    cudaGraphExec_t realizeGraph = nullptr;  // captured after tuning
    // tree operators (allocated on first use): FP64 scratch for a batch whose
    // own scratch is FP32, device operands and results in the host packing,
    // their pinned host staging, and the per-instance packing offsets
    void* opsScratch = nullptr;
    double* opsDev = nullptr;
    double* opsHost = nullptr;
    int64_t opsElems = 0;
    int64_t* dHostBOff = nullptr;
    cudaEvent_t evOp0 = nullptr, evOp1 = nullptr;  // bracket the last tree operator's kernels
    // one-step launches of a mixed batch integration (allocated on first use)
    std::vector<int64_t> rowsElems;   // FP64 level-parallel record elements per instance (0: loop closures)
    int32_t* fbList = nullptr;        // 2 x ninst
    int32_t* fbCount = nullptr;       // 2, then the unfinished count
    int32_t* fbMode = nullptr;        // 2 x ninst
    int32_t* fbLeft = nullptr;
    int32_t* stepsLeft = nullptr;
    int64_t fbLaunch = 0;             // one-step launches of the integration so far (continued calls go on)
    bool fbAllFp64 = false;           // the integration switched to the FP64 kernels (too many FP64 steps)
    unsigned long long fbWindow0 = 0; // FP64 steps counted at the start of the current window
    double* fbuf64 = nullptr;
    unsigned long long* fbSteps = nullptr;
    long long* adaptStats = nullptr;  // accepted / rejected steps of the error-controlled integrator
    int64_t* rowsBase = nullptr;
    double* rows = nullptr;
    cudaStream_t fbStream = nullptr;
    cudaEvent_t fbFork = nullptr, fbJoin = nullptr;

    Streams streams() const { return Streams{stream, stream2, evFork, evJoin}; }
    LaunchPlan plan() const { return LaunchPlan{nChain, nGroupBlocks, nm, variant == 0 ? 1 : variant, nLoop}; }
    BatchBufs bufsArg() const { return BatchBufs{scratch, scratchLoop, fbuf, fbufLoop, colElems}; }
    int segments() const { return (nChain > 0) + (nLoop > 0) + (nGroupBlocks > 0); }
    // kernels of one realize: the segments, and in the mixed form the FP64
    // recomputation pass after the chain and the level-parallel segment
    int realizeLaunches() const {
        return segments() + (T.scratch64 ? (nChain > 0) + (nGroupBlocks > 0) : 0);
    }

    // Lanes per instance of the group segment: blocks of 128 threads hold
    // 128/G instances of equal G (the order is sorted by widest level, so G is
    // non-increasing along it).
    int setGroupShift(int shift) {
        if (shift == groupShift) return SBG_OK;
        std::vector<int32_t> first, gs;
        const int ng = (int)groupWidthKey.size();
        int p = 0;
        while (p < ng) {
            int w = 1;
            while (w < groupWidthKey[p]) w <<= 1;
            const int G = std::max(2, std::min(32, w >> shift));
            int q = p;
            auto gOf = [&](int k) { int ww = 1; while (ww < groupWidthKey[k]) ww <<= 1; return std::max(2, std::min(32, ww >> shift)); };
            while (q < ng && q - p < 128 / G && gOf(q) == G) ++q;
            first.push_back(nChain + nLoop + p);
            gs.push_back(G);
            p = q;
        }
        first.push_back(nChain + nLoop + ng);
        gs.push_back(0);
        nGroupBlocks = (int)gs.size() - 1;
        cudaError_t e = cudaMemcpy(dBlkFirst, first.data(), first.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(dBlkG, gs.data(), gs.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cudaFail(e, "group block table");
        groupShift = shift;
        return SBG_OK;
    }

    ~sbg_batch_s() {
        if (device >= 0) cudaSetDevice(device);
        for (auto& b : bufs) cudaFree(b.p);
        if (hostPinned) cudaFreeHost(hostPinned);
        if (opsHost) cudaFreeHost(opsHost);
        if (realizeGraph) cudaGraphExecDestroy(realizeGraph);
        if (evFork) cudaEventDestroy(evFork);
        if (evT0) cudaEventDestroy(evT0);
        if (evT1) cudaEventDestroy(evT1);
        if (evOp0) cudaEventDestroy(evOp0);
        if (evOp1) cudaEventDestroy(evOp1);
        if (evJoin) cudaEventDestroy(evJoin);
        if (fbFork) cudaEventDestroy(fbFork);
        if (fbJoin) cudaEventDestroy(fbJoin);
        if (fbStream) cudaStreamDestroy(fbStream);
        if (stream2) cudaStreamDestroy(stream2);
        for (int k = 1; k < 5; ++k)
            if (pipe[k]) cudaStreamDestroy(pipe[k]);
        for (auto& row : pipeEv)
            for (cudaEvent_t e : row)
                if (e) cudaEventDestroy(e);
        if (pipeStart) cudaEventDestroy(pipeStart);
        if (pipeEnd) cudaEventDestroy(pipeEnd);
        if (stream) cudaStreamDestroy(stream);
    }
    int alloc(void** out, size_t bytes, const char* what) {
        if (budget > 0 && devBytes + (int64_t)bytes > budget)
            return fail(SBG_ERR_BUDGET, std::string("device budget exceeded allocating ") + what);
        void* p = nullptr;
        if (bytes) {
            cudaError_t e = cudaMalloc(&p, bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(SBG_ERR_NOMEM, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
            }
        }
        bufs.push_back({p, bytes});
        devBytes += (int64_t)bytes;
        *out = p;
        return SBG_OK;
    }
    template <class T_> int upload(const T_** dst, const std::vector<T_>& v, const char* what) {
        void* p = nullptr;
        int rc = alloc(&p, v.size() * sizeof(T_), what);
        if (rc) return rc;
        if (!v.empty()) {
            cudaError_t e = cudaMemcpy(p, v.data(), v.size() * sizeof(T_), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return cudaFail(e, what);
        }
        *dst = static_cast<const T_*>(p);
        return SBG_OK;
    }
};

extern "C" {

const char* sbg_last_error(void) { return g_err.c_str(); }
int sbg_abi_version(void) { return SBG_ABI_VERSION; }
int sbg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// ------------------------------------------------------------------ topology
int sbg_topology_create(const sbg_system_desc* d, sbg_topology* out) {
    if (!d || !out) return fail(SBG_ERR_INVALID, "null argument");
    if (d->nbodies < 1 || !d->bodies) return fail(SBG_ERR_INVALID, "system has no bodies");
    if (d->nforces < 0 || (d->nforces > 0 && !d->forces)) return fail(SBG_ERR_INVALID, "bad force list");
    if (d->nconstraints < 0 || (d->nconstraints > 0 && !d->constraints))
        return fail(SBG_ERR_INVALID, "bad constraint list");
    if (d->flags & ~SBG_SYSTEM_EULER_ANGLES) return fail(SBG_ERR_INVALID, "unknown system flags");
    const bool euler = (d->flags & SBG_SYSTEM_EULER_ANGLES) != 0;
    const int nb = d->nbodies;
    std::vector<int> level(nb + 1, 0), qo(nb + 1, 0), uo(nb + 1, 0);
    int nq = 0, nu = 0, nquat = 0, maxnf = 0;
    auto isQuat = [&](int mob) { return !euler && (mob == SBG_BALL || mob == SBG_FREE); };
    for (int i = 1; i <= nb; ++i) {
        const sbg_body_desc& b = d->bodies[i - 1];
        if (b.parent < 0 || b.parent >= i)
            return fail(SBG_ERR_INVALID, "body " + std::to_string(i) + ": parent must precede the body");
        if (b.mobilizer < 0 || b.mobilizer >= SBG_NUM_MOBILIZERS)
            return fail(SBG_ERR_INVALID, "body " + std::to_string(i) + ": unknown mobilizer");
        if (!(b.mass > 0) || !std::isfinite(b.mass))
            return fail(SBG_ERR_INVALID, "body " + std::to_string(i) + ": mass must be positive and finite");
        level[i] = level[b.parent] + 1;
        qo[i] = nq;
        uo[i] = nu;
        nq += kNQ[b.mobilizer];
        nu += kNU[b.mobilizer];
        if (isQuat(b.mobilizer)) ++nquat;
        if (kNU[b.mobilizer] != 6) maxnf = std::max(maxnf, kNU[b.mobilizer]);  // 6-mobility rows have their own width
    }
    for (int i = 0; i < d->nforces; ++i) {
        const auto& f = d->forces[i];
        if (f.body < 1 || f.body > nb) return fail(SBG_ERR_INVALID, "mobility force on a bad body");
        if (f.kind != 0 && f.kind != 1) return fail(SBG_ERR_INVALID, "unknown mobility force kind");
        if (f.which < 0 || f.which >= kNU[d->bodies[f.body - 1].mobilizer])
            return fail(SBG_ERR_INVALID, "mobility index out of range");
    }
    for (int i = 0; i < d->nconstraints; ++i) {
        const auto& c = d->constraints[i];
        if (c.body1 < 0 || c.body1 > nb || c.body2 < 0 || c.body2 > nb || c.body1 == c.body2)
            return fail(SBG_ERR_INVALID, "Ball constraint on bad bodies");
    }
    if (d->ncontacts < 0 || (d->ncontacts > 0 && !d->contacts)) return fail(SBG_ERR_INVALID, "bad contact list");
    for (int i = 0; i < d->ncontacts; ++i) {
        const auto& k = d->contacts[i];
        if (k.body < 1 || k.body > nb) return fail(SBG_ERR_INVALID, "contact sphere on a bad body");
        if (!(k.radius > 0) || !std::isfinite(k.radius))
            return fail(SBG_ERR_INVALID, "contact sphere radius must be positive and finite");
    }
    auto* t = new (std::nothrow) sbg_topology_s();
    if (!t) return fail(SBG_ERR_NOMEM, "out of host memory");
    t->nb = nb;
    t->nq = nq;
    t->nu = nu;
    t->nquat = nquat;
    t->ncons = d->nconstraints;
    t->ncontacts = d->ncontacts;
    t->maxNonFreeDof = maxnf;
    for (int k = 0; k < 3; ++k) t->gravity[k] = d->gravity[k];
    // level order: stable sort of bodies by level
    std::vector<int> order(nb);
    std::iota(order.begin(), order.end(), 1);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return level[a] < level[b]; });
    std::vector<int> rowOf(nb + 1, -1);
    for (int r = 0; r < nb; ++r) rowOf[order[r]] = r;
    t->nlevels = level[order.back()];
    // forces grouped by body, application order preserved
    std::vector<std::vector<int>> fOf(nb + 1);
    for (int i = 0; i < d->nforces; ++i) fOf[d->forces[i].body].push_back(i);
    std::vector<std::vector<int>> kOf(nb + 1);
    for (int i = 0; i < d->ncontacts; ++i) kOf[d->contacts[i].body].push_back(i);
    std::vector<std::vector<int>> kids(nb + 1);
    for (int i = 1; i <= nb; ++i) kids[d->bodies[i - 1].parent].push_back(i);
    // bodies on the way from a loop body to Ground
    std::vector<char> onLoopPath(nb + 1, 0);
    for (int i = 0; i < d->nconstraints; ++i)
        for (int b : {d->constraints[i].body1, d->constraints[i].body2})
            for (int k = b; k > 0 && !onLoopPath[k]; k = d->bodies[k - 1].parent) onLoopPath[k] = 1;
    int64_t rec = 0;
    for (int r = 0; r < nb; ++r) {
        const int bi = order[r];
        const sbg_body_desc& b = d->bodies[bi - 1];
        const int n = kNU[b.mobilizer];
        int info = b.mobilizer | (n << 4);
        if (isIdentityR(b.X_PF)) info |= 1 << 8;
        if (isIdentityR(b.X_BM)) info |= 1 << 9;
        if (b.X_BM[9] == 0 && b.X_BM[10] == 0 && b.X_BM[11] == 0) info |= 1 << 10;
        if (b.X_PF[9] == 0 && b.X_PF[10] == 0 && b.X_PF[11] == 0) info |= 1 << 11;
        if (b.parent != 0 && rowOf[b.parent] == r - 1) info |= F_CARRY;
        for (int c : kids[bi])
            if (rowOf[c] != r + 1) info |= F_MEMCHILD;
        for (int i = 0; i < d->nconstraints; ++i)
            if (d->constraints[i].body1 == bi || d->constraints[i].body2 == bi) info |= F_LOOPBODY;
        if (onLoopPath[bi]) info |= F_LOOPPATH;
        if (isQuat(b.mobilizer)) info |= F_QUAT;
        if (!kOf[bi].empty()) info |= F_CONTACT;
        t->parent.push_back(b.parent == 0 ? -1 : rowOf[b.parent]);
        t->info.push_back(info);
        t->qoff.push_back(qo[bi]);
        t->uoff.push_back(uo[bi]);
        t->srec.push_back((int32_t)rec);
        t->bodyOfRow.push_back(bi - 1);
        rec += scratchRecordSize(n);
        t->fbeg.push_back((int32_t)t->fkw.size());
        t->fcnt.push_back((int32_t)fOf[bi].size());
        for (int fi : fOf[bi]) {
            const auto& f = d->forces[fi];
            t->fkw.push_back((f.kind << 8) | f.which);
            t->fcoef.push_back(f.coef);
            t->fq0.push_back(f.q0);
        }
        t->kbeg.push_back((int32_t)t->kpar.size());
        t->kcnt.push_back((int32_t)kOf[bi].size());
        for (int ki : kOf[bi]) {
            const sbg_contact_desc& k = d->contacts[ki];
            double c[kContactStride];
            for (int j = 0; j < 3; ++j) c[j] = k.station[j];
            c[3] = k.radius;
            for (int j = 0; j < 3; ++j) c[4 + j] = k.halfspace[3 * j];  // x axis of the half-space frame
            for (int j = 0; j < 3; ++j) c[7 + j] = k.halfspace[9 + j];
            // parameters, the reference's defaults for an all-zero block
            // (SmoothSphereHalfSpaceForceImpl::Parameters())
            double stiff = k.stiffness, diss = k.dissipation, us = k.static_friction, ud = k.dynamic_friction,
                   uv = k.viscous_friction, vt = k.transition_velocity, cf = k.cf, bd = k.bd, bv = k.bv;
            if (stiff == 0 && diss == 0 && us == 0 && ud == 0 && uv == 0 && vt == 0 && cf == 0 && bd == 0 && bv == 0) {
                stiff = 1; vt = 0.01; cf = 1e-5; bd = 300; bv = 50;
            }
            const double kk = 0.5 * std::pow(stiff, 2.0 / 3.0);
            c[10] = (4.0 / 3.0) * kk * std::sqrt(k.radius * kk);
            c[11] = diss; c[12] = us; c[13] = ud; c[14] = uv; c[15] = vt; c[16] = cf; c[17] = bd; c[18] = bv;
            c[19] = 2.0 / (3.0 * diss);
            t->kpar.insert(t->kpar.end(), c, c + kContactStride);
        }
        // params: mass, com, G, R_PF, p_PF, R_MB = ~R_BM, p_MB = -(~R_BM p_BM), pitch
        double p[kParamStride];
        p[0] = b.mass;
        for (int k = 0; k < 3; ++k) p[1 + k] = b.com[k];
        for (int k = 0; k < 6; ++k) p[4 + k] = b.unit_inertia[k];
        for (int k = 0; k < 9; ++k) p[10 + k] = b.X_PF[k];
        for (int k = 0; k < 3; ++k) p[19 + k] = b.X_PF[9 + k];
        for (int r2 = 0; r2 < 3; ++r2)
            for (int c = 0; c < 3; ++c) p[22 + 3 * r2 + c] = b.X_BM[3 * c + r2];
        for (int r2 = 0; r2 < 3; ++r2)
            p[31 + r2] = -(p[22 + 3 * r2] * b.X_BM[9] + p[22 + 3 * r2 + 1] * b.X_BM[10] + p[22 + 3 * r2 + 2] * b.X_BM[11]);
        p[34] = b.mobilizer == SBG_SCREW ? b.pitch : 0.0;
        t->par.insert(t->par.end(), p, p + kParamStride);
    }
    t->recSize = rec;
    // level table, children lists and shape of the tree (local rows)
    t->levStart.assign(t->nlevels + 1, nb);
    for (int r = nb - 1; r >= 0; --r) t->levStart[level[order[r]] - 1] = r;
    t->levStart[t->nlevels] = nb;
    for (int L = 0; L < t->nlevels; ++L) t->maxLevelWidth = std::max(t->maxLevelWidth, t->levStart[L + 1] - t->levStart[L]);
    t->cbeg.assign(nb, 0);
    t->ccnt.assign(nb, 0);
    for (int r = 0; r < nb; ++r)
        if (t->parent[r] >= 0) ++t->ccnt[t->parent[r]];
    for (int r = 1; r < nb; ++r) t->cbeg[r] = t->cbeg[r - 1] + t->ccnt[r - 1];
    t->clist.assign(nb > 0 ? t->cbeg[nb - 1] + t->ccnt[nb - 1] : 0, 0);
    {
        std::vector<int32_t> fill(t->cbeg);
        for (int r = 0; r < nb; ++r)
            if (t->parent[r] >= 0) t->clist[fill[t->parent[r]]++] = r;
    }
    t->chain = true;
    for (int r = 0; r < nb; ++r)
        if (t->parent[r] != r - 1) t->chain = false;
    t->defaultY.assign(nq + nu, 0.0);
    for (int i = 1; i <= nb; ++i)
        if (isQuat(d->bodies[i - 1].mobilizer)) t->defaultY[qo[i]] = 1.0;
    for (int i = 0; i < d->nconstraints; ++i) t->cons.push_back(d->constraints[i]);
    t->lslot.assign(nb, -1);
    for (int r = 0; r < nb; ++r)
        if (t->info[r] & F_LOOPBODY) t->lslot[r] = t->nslots++;
    for (const auto& c : t->cons) {
        t->lcons.push_back(c.body1 == 0 ? -1 : rowOf[c.body1]);
        t->lcons.push_back(c.body2 == 0 ? -1 : rowOf[c.body2]);
        t->lst.insert(t->lst.end(), c.station1, c.station1 + 3);
        t->lst.insert(t->lst.end(), c.station2, c.station2 + 3);
    }
    *out = t;
    return SBG_OK;
}

int sbg_topology_destroy(sbg_topology t) {
    delete t;
    return SBG_OK;
}

int sbg_topology_info(sbg_topology t, int32_t* nq, int32_t* nu, int32_t* nbodies, int32_t* nlevels,
                      int32_t* nquaternions, int32_t* ncons) {
    if (!t) return fail(SBG_ERR_INVALID, "null topology");
    if (nq) *nq = t->nq;
    if (nu) *nu = t->nu;
    if (nbodies) *nbodies = t->nb;
    if (nlevels) *nlevels = t->nlevels;
    if (nquaternions) *nquaternions = t->nquat;
    if (ncons) *ncons = 3 * t->ncons;
    return SBG_OK;
}

int sbg_topology_default_state(sbg_topology t, double* y) {
    if (!t || !y) return fail(SBG_ERR_INVALID, "null argument");
    std::copy(t->defaultY.begin(), t->defaultY.end(), y);
    return SBG_OK;
}

// --------------------------------------------------------------------- batch
int sbg_batch_create(const sbg_topology* topos, int32_t ntopo, const int32_t* instTopo, int32_t ninst,
                     const sbg_batch_config* cfg, sbg_batch* out) {
    if (!topos || ntopo < 1 || !instTopo || ninst < 0 || !out) return fail(SBG_ERR_INVALID, "bad batch arguments");
    const int precision = cfg ? cfg->precision : SBG_PRECISION_FP64;
    if (precision != SBG_PRECISION_FP64 && precision != SBG_PRECISION_MIXED && precision != SBG_PRECISION_MIXED_FAST)
        return fail(SBG_ERR_INVALID, "unknown precision");
    for (int i = 0; i < ninst; ++i)
        if (instTopo[i] < 0 || instTopo[i] >= ntopo || !topos[instTopo[i]])
            return fail(SBG_ERR_INVALID, "instance " + std::to_string(i) + " names a bad topology");
    for (int k = 0; k < ntopo; ++k)
        if (topos[k] && topos[k]->ncons > kMaxLoopCons)
            return fail(SBG_ERR_UNSUPPORTED, "at most " + std::to_string(kMaxLoopCons) +
                                                 " Ball loop closures per system are supported");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SBG_ERR_NO_DEVICE, "no CUDA device available");
    }
    const int device = cfg ? cfg->device : 0;
    if (device < 0 || device >= ndev) return fail(SBG_ERR_INVALID, "bad device ordinal");
    SBG_CUDA(cudaSetDevice(device), "cudaSetDevice");

    auto* b = new (std::nothrow) sbg_batch_s();
    if (!b) return fail(SBG_ERR_NOMEM, "out of host memory");
    b->precision = precision;
    b->device = device;
    b->budget = cfg ? cfg->device_budget_bytes : 0;
    b->ninst = ninst;
    b->instTopo.assign(instTopo, instTopo + ninst);
    auto bail = [&](int rc) { delete b; return rc; };
    {
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream2, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->evFork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->evJoin, cudaEventDisableTiming);
        if (e != cudaSuccess) return bail(cudaFail(e, "stream/event creation"));
    }

    // batch width: 1 when every non-Free body has one mobility, else 3
    int nm = 1;
    for (int i = 0; i < ninst; ++i)
        if (topos[instTopo[i]]->maxNonFreeDof > 1) nm = 3;
    // distinct topologies used, concatenated body tables
    std::vector<int> used(ntopo, -1);
    std::vector<int64_t> recTotal(ntopo, 0);
    std::vector<int32_t> parent, info, qoff, uoff, srec, fbeg, fcnt, fkw, bidx, kbeg, kcnt;
    std::vector<double> par, fcoef, fq0, kpar;
    std::vector<int32_t> rowBase(ntopo, 0);
    for (int i = 0; i < ninst; ++i) {
        const int k = instTopo[i];
        if (used[k] >= 0) continue;
        used[k] = 1;
        const sbg_topology_s* t = topos[k];
        rowBase[k] = (int32_t)parent.size();
        const int32_t fOff = (int32_t)fkw.size();
        parent.insert(parent.end(), t->parent.begin(), t->parent.end());
        info.insert(info.end(), t->info.begin(), t->info.end());
        qoff.insert(qoff.end(), t->qoff.begin(), t->qoff.end());
        uoff.insert(uoff.end(), t->uoff.begin(), t->uoff.end());
        bidx.insert(bidx.end(), t->bodyOfRow.begin(), t->bodyOfRow.end());
        const std::vector<int32_t> pr = paddedRecords(*t, nm, &recTotal[k]);
        srec.insert(srec.end(), pr.begin(), pr.end());
        for (int32_t fb : t->fbeg) fbeg.push_back(fb + fOff);
        fcnt.insert(fcnt.end(), t->fcnt.begin(), t->fcnt.end());
        fkw.insert(fkw.end(), t->fkw.begin(), t->fkw.end());
        fcoef.insert(fcoef.end(), t->fcoef.begin(), t->fcoef.end());
        fq0.insert(fq0.end(), t->fq0.begin(), t->fq0.end());
        const int32_t kOff = (int32_t)kpar.size();
        for (int32_t kb : t->kbeg) kbeg.push_back(kb + kOff);
        kcnt.insert(kcnt.end(), t->kcnt.begin(), t->kcnt.end());
        kpar.insert(kpar.end(), t->kpar.begin(), t->kpar.end());
        par.insert(par.end(), t->par.begin(), t->par.end());
    }
    b->nm = nm;
    const bool uniform = ninst > 0 && std::all_of(instTopo, instTopo + ninst, [&](int32_t k) { return k == instTopo[0]; });

    // Instance table and column addressing.
    //  - chain segment (order positions [0, nChain)): chains and near-chains,
    //    one thread per instance, largest first; 32 consecutive positions form
    //    a tile whose state columns and scratch records interleave lane by
    //    lane (element e of the lane-l instance at tileBase + e*32 + l),
    //    padded to the tile's largest instance;
    //  - group segment (the rest): trees with wide levels, G lanes per
    //    instance; each instance's state is contiguous and its scratch is
    //    field-major (element f of row r at base + r + f*nbodies).
    std::vector<int32_t> ibody(ninst), inb(ninst), inq(ninst), inu(ninst), order(ninst), ilev(ninst), inlev(ninst);
    std::vector<int64_t> ybase(ninst), ystride(ninst), sbase(ninst), sstride(ninst);
    std::vector<double> grav(3 * (size_t)ninst);
    std::vector<int32_t> levBase(ntopo, 0);
    std::vector<int32_t> levStart, cbeg, ccnt, clist;
    for (int k = 0; k < ntopo; ++k) {
        if (used[k] < 0) continue;
        const sbg_topology_s* t = topos[k];
        levBase[k] = (int32_t)levStart.size();
        levStart.insert(levStart.end(), t->levStart.begin(), t->levStart.end());
        const int32_t cOff = (int32_t)clist.size();
        for (int32_t v : t->cbeg) cbeg.push_back(v + cOff);
        ccnt.insert(ccnt.end(), t->ccnt.begin(), t->ccnt.end());
        clist.insert(clist.end(), t->clist.begin(), t->clist.end());
    }
    b->hostYOff.assign(ninst + 1, 0);
    b->hostUOff.assign(ninst + 1, 0);
    b->hostBOff.assign(ninst + 1, 0);
    // Trees with fewer bodies run one per thread (their lanes would mostly
    // idle or diverge in a group); larger trees with wide levels get a group.
    int groupMinBodies = 48;
    if (const char* v = std::getenv("SBG_GROUP_MIN_BODIES")) groupMinBodies = std::atoi(v);  // tuning override
    std::vector<int> chainPos, loopPos, groupPos;
    for (int i = 0; i < ninst; ++i) {
        const sbg_topology_s* t = topos[instTopo[i]];
        ibody[i] = rowBase[instTopo[i]];
        inb[i] = t->nb;
        inq[i] = t->nq;
        inu[i] = t->nu;
        ilev[i] = levBase[instTopo[i]];
        inlev[i] = t->nlevels;
        for (int k = 0; k < 3; ++k) grav[3 * i + k] = t->gravity[k];
        b->hostYOff[i + 1] = b->hostYOff[i] + t->nq + t->nu;
        b->hostUOff[i + 1] = b->hostUOff[i] + t->nu;
        b->hostBOff[i + 1] = b->hostBOff[i] + t->nb;
        b->rowsElems.push_back(t->ncons > 0 ? 0 : (int64_t)t->nb * rowsRecordWidth(*t, 3));
        if (t->ncons > 0) loopPos.push_back(i);
        else if (t->chain || t->maxLevelWidth <= 2 || t->nb < groupMinBodies) chainPos.push_back(i);
        else groupPos.push_back(i);
    }
    if (!uniform) {
        std::stable_sort(chainPos.begin(), chainPos.end(), [&](int a, int c) { return inb[a] > inb[c]; });
        std::stable_sort(loopPos.begin(), loopPos.end(), [&](int a, int c) { return inb[a] > inb[c]; });
        auto wkey = [&](int i) { int w = 1; while (w < topos[instTopo[i]]->maxLevelWidth) w <<= 1; return w; };
        std::stable_sort(groupPos.begin(), groupPos.end(), [&](int a, int c) {
            const int wa = wkey(a), wc = wkey(c);
            return wa != wc ? wa > wc : inb[a] > inb[c];
        });
    }
    b->nChain = (int)chainPos.size();
    b->nLoop = (int)loopPos.size();
    b->orderIdentity = b->nChain == ninst;
    for (int i = 0; i < b->nChain && b->orderIdentity; ++i) b->orderIdentity = chainPos[i] == i;
    std::copy(chainPos.begin(), chainPos.end(), order.begin());
    std::copy(loopPos.begin(), loopPos.end(), order.begin() + b->nChain);
    std::copy(groupPos.begin(), groupPos.end(), order.begin() + b->nChain + b->nLoop);
    // slot records of the loop-closure topologies follow their body records
    std::vector<int32_t> lrec(parent.size(), -1), lslot(parent.size(), -1);
    for (int k = 0; k < ntopo; ++k) {
        if (used[k] < 0) continue;
        const sbg_topology_s* t = topos[k];
        for (int r = 0; r < t->nb; ++r)
            if (t->lslot[r] >= 0) {
                lrec[rowBase[k] + r] = (int32_t)(recTotal[k] + (int64_t)t->lslot[r] * kSlotSize);
                lslot[rowBase[k] + r] = t->lslot[r];
            }
    }
    int64_t yOff = 0, sOff = 0, sOffLoop = 0;
    // tiles of 32 chain-driver instances (the chain segment, then the
    // loop-closure segment with its own FP64 scratch)
    auto tile = [&](int p0, int p1, int64_t& sOffSeg, bool loops) {
        for (int t0 = p0; t0 < p1; t0 += kTile) {
            const int t1 = std::min(p1, t0 + kTile);
            int64_t yw = 0, sw = 0;
            for (int p = t0; p < t1; ++p) {
                const int i = order[p];
                const sbg_topology_s* t = topos[instTopo[i]];
                yw = std::max<int64_t>(yw, inq[i] + inu[i]);
                sw = std::max<int64_t>(sw, recTotal[instTopo[i]] + (loops ? (int64_t)t->nslots * kSlotSize : 0));
            }
            for (int p = t0; p < t1; ++p) {
                const int i = order[p];
                ybase[i] = yOff + (p - t0); ystride[i] = kTile;
                sbase[i] = sOffSeg + (p - t0); sstride[i] = kTile;
            }
            yOff += yw * kTile;
            sOffSeg += sw * kTile;
        }
    };
    tile(0, b->nChain, sOff, false);
    tile(b->nChain, b->nChain + b->nLoop, sOffLoop, true);
    // constraint tables
    std::vector<int32_t> lcons, icons(ninst, 0), incons(ninst, 0), consBase(ntopo, 0);
    std::vector<double> lst;
    for (int k = 0; k < ntopo; ++k) {
        if (used[k] < 0) continue;
        consBase[k] = (int32_t)(lcons.size() / 2);
        lcons.insert(lcons.end(), topos[k]->lcons.begin(), topos[k]->lcons.end());
        lst.insert(lst.end(), topos[k]->lst.begin(), topos[k]->lst.end());
    }
    for (int i = 0; i < ninst; ++i) {
        icons[i] = consBase[instTopo[i]];
        incons[i] = topos[instTopo[i]]->ncons;
    }
    b->groupWidthKey.clear();
    for (int p = b->nChain + b->nLoop; p < ninst; ++p) {
        const int i = order[p];
        const sbg_topology_s* t = topos[instTopo[i]];
        ybase[i] = yOff; ystride[i] = 1;
        yOff += t->nq + t->nu;
        sbase[i] = sOff; sstride[i] = 1;
        sOff += (int64_t)t->nb * rowsRecordWidth(*t, 3);
        b->groupWidthKey.push_back(t->maxLevelWidth);
    }
    b->nyTotal = b->hostYOff[ninst];
    b->nuTotal = b->hostUOff[ninst];
    b->colElems = yOff;
    b->scratchElems = sOff;
    const int64_t scratchLoopElems = sOffLoop;
    b->tiled = true;
    {
        int nUsed = 0, k0 = -1;
        for (int k = 0; k < ntopo; ++k)
            if (used[k] >= 0) { ++nUsed; k0 = k; }
        bool ok = nUsed == 1 && precision != SBG_PRECISION_FP64 && b->nChain == ninst && topos[k0]->chain;
        for (int r = 0; ok && r < topos[k0]->nb; ++r)
            if (((topos[k0]->info[r] >> 4) & 15) == 6) ok = false;
        b->stagedOk = ok;
    }
    if (precision == SBG_PRECISION_FP64) b->variant = 1;  // FP64 needs every register
    if (const char* v = std::getenv("SBG_VARIANT")) {  // tuning override
        const int want = std::atoi(v);
        b->variant = want == 8 ? (b->stagedOk ? 8 : 7) : want == 4 || want == 7 ? want : 1;
    }

    int rc = 0;
    DevTables& T = b->T;
    T.ninst = ninst;
    std::vector<float> par32(par.begin(), par.end()), fcoef32(fcoef.begin(), fcoef.end()), fq032(fq0.begin(), fq0.end());
    if ((rc = b->upload(&T.parent, parent, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.info, info, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.qoff, qoff, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.uoff, uoff, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.srec, srec, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.bidx, bidx, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.fbeg, fbeg, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.fcnt, fcnt, "body table"))) return bail(rc);
    if ((rc = b->upload(&T.par64, par, "parameters"))) return bail(rc);
    if ((rc = b->upload(&T.par32, par32, "parameters"))) return bail(rc);
    if ((rc = b->upload(&T.fkind_which, fkw, "force table"))) return bail(rc);
    if ((rc = b->upload(&T.fcoef64, fcoef, "force table"))) return bail(rc);
    if ((rc = b->upload(&T.fq064, fq0, "force table"))) return bail(rc);
    if ((rc = b->upload(&T.fcoef32, fcoef32, "force table"))) return bail(rc);
    if ((rc = b->upload(&T.fq032, fq032, "force table"))) return bail(rc);
    if (!kpar.empty()) {
        const std::vector<float> kpar32(kpar.begin(), kpar.end());
        if ((rc = b->upload(&T.kbeg, kbeg, "contact table"))) return bail(rc);
        if ((rc = b->upload(&T.kcnt, kcnt, "contact table"))) return bail(rc);
        if ((rc = b->upload(&T.kpar64, kpar, "contact table"))) return bail(rc);
        if ((rc = b->upload(&T.kpar32, kpar32, "contact table"))) return bail(rc);
    }
    if ((rc = b->upload(&T.ibody, ibody, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.inb, inb, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.inq, inq, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.inu, inu, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.ybase, ybase, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.ystride, ystride, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.sbase, sbase, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.sstride, sstride, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.grav, grav, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.order, order, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.ilev, ilev, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.inlev, inlev, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.levStart, levStart, "level table"))) return bail(rc);
    if ((rc = b->upload(&T.cbeg, cbeg, "children table"))) return bail(rc);
    if ((rc = b->upload(&T.ccnt, ccnt, "children table"))) return bail(rc);
    if ((rc = b->upload(&T.clist, clist, "children table"))) return bail(rc);
    if ((rc = b->upload(&T.lrec, lrec, "loop table"))) return bail(rc);
    if ((rc = b->upload(&T.lslot, lslot, "loop table"))) return bail(rc);
    if ((rc = b->upload(&T.lcons, lcons, "loop table"))) return bail(rc);
    if ((rc = b->upload(&T.lst, lst, "loop table"))) return bail(rc);
    if ((rc = b->upload(&T.icons, icons, "instance table"))) return bail(rc);
    if ((rc = b->upload(&T.incons, incons, "instance table"))) return bail(rc);
    {   // group block table (capacity: one block per group instance + end)
        void* q = nullptr;
        const size_t cap = (size_t)(ninst - b->nChain - b->nLoop) + 2;
        if ((rc = b->alloc(&q, cap * sizeof(int32_t), "group block table"))) return bail(rc);
        b->dBlkFirst = static_cast<int32_t*>(q);
        if ((rc = b->alloc(&q, cap * sizeof(int32_t), "group block table"))) return bail(rc);
        b->dBlkG = static_cast<int32_t*>(q);
        T.blkFirst = b->dBlkFirst;
        T.blkG = b->dBlkG;
        if ((rc = b->setGroupShift(1))) return bail(rc);
    }
    const int64_t* dOff = nullptr;
    if ((rc = b->upload(&dOff, b->hostYOff, "offsets"))) return bail(rc);
    b->dHostYOff = const_cast<int64_t*>(dOff);
    if ((rc = b->upload(&dOff, b->hostUOff, "offsets"))) return bail(rc);
    b->dHostUOff = const_cast<int64_t*>(dOff);
    {
        std::vector<int64_t> qo(ninst + 1);
        for (int i = 0; i <= ninst; ++i) qo[i] = b->hostYOff[i] - b->hostUOff[i];
        if ((rc = b->upload(&dOff, qo, "offsets"))) return bail(rc);
        b->dHostQOff = const_cast<int64_t*>(dOff);
    }

    const size_t rsz = precision == SBG_PRECISION_FP64 ? sizeof(double) : sizeof(float);
    void* p = nullptr;
    if ((rc = b->alloc(&p, b->colElems * sizeof(double), "state"))) return bail(rc);
    b->y = static_cast<double*>(p);
    if ((rc = b->alloc(&p, b->colElems * sizeof(double), "derivatives"))) return bail(rc);
    b->ydot = static_cast<double*>(p);
    if ((rc = b->alloc(&p, b->colElems * sizeof(double), "M^-1 input"))) return bail(rc);
    b->fcol = static_cast<double*>(p);
    if ((rc = b->alloc(&p, std::max<int64_t>(ninst, 1) * sizeof(double), "time"))) return bail(rc);
    b->time = static_cast<double*>(p);
    if ((rc = b->alloc(&p, std::max<int64_t>(ninst, 1) * sizeof(int32_t), "status"))) return bail(rc);
    b->status = static_cast<int32_t*>(p);
    if ((rc = b->alloc(&p, std::max<int64_t>(b->nyTotal, 1) * sizeof(double), "staging"))) return bail(rc);
    b->staging = static_cast<double*>(p);
    if ((rc = b->alloc(&b->scratch, std::max<int64_t>(b->scratchElems, 1) * rsz, "scratch"))) return bail(rc);
    if (precision == SBG_PRECISION_MIXED && b->scratchElems > 0) {
        // FP64 mirror of the scratch for the instances whose refinement
        // reports an ill-conditioned M, and the count of those recomputed
        if ((rc = b->alloc(&p, b->scratchElems * sizeof(double), "FP64 scratch mirror"))) return bail(rc);
        T.scratch64 = static_cast<double*>(p);
        if ((rc = b->alloc(&p, sizeof(unsigned long long), "fallback counter"))) return bail(rc);
        T.fallbacks = static_cast<unsigned long long*>(p);
        const cudaError_t ez = cudaMemset(p, 0, sizeof(unsigned long long));
        if (ez != cudaSuccess) return bail(cudaFail(ez, "fallback counter"));
    }
    if ((rc = b->alloc(&b->fbuf, 4 * std::max<int64_t>(b->colElems, 1) * rsz, "stage derivatives"))) return bail(rc);
    if (b->nLoop > 0) {
        if ((rc = b->alloc(&b->scratchLoop, scratchLoopElems * sizeof(double), "loop scratch"))) return bail(rc);
        if (precision == SBG_PRECISION_FP64) b->fbufLoop = b->fbuf;
        else if ((rc = b->alloc(&b->fbufLoop, 4 * b->colElems * sizeof(double), "loop stage derivatives")))
            return bail(rc);
    }
    {
        cudaError_t e = cudaMallocHost(&b->hostPinned, std::max<int64_t>(b->nyTotal, 1) * sizeof(double));
        if (e != cudaSuccess) return bail(cudaFail(e, "cudaMallocHost"));
    }
    cudaError_t e = cudaMemsetAsync(b->time, 0, std::max<int64_t>(ninst, 1) * sizeof(double), b->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->status, 0, std::max<int64_t>(ninst, 1) * sizeof(int32_t), b->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
    if (e != cudaSuccess) return bail(cudaFail(e, "batch initialisation"));
    *out = b;
    return SBG_OK;
}

int sbg_batch_destroy(sbg_batch b) {
    delete b;
    return SBG_OK;
}

int sbg_batch_layout(sbg_batch b, int64_t* yOff, int64_t* nyTotal) {
    if (!b) return fail(SBG_ERR_INVALID, "null batch");
    if (yOff) std::copy(b->hostYOff.begin(), b->hostYOff.end(), yOff);
    if (nyTotal) *nyTotal = b->nyTotal;
    return SBG_OK;
}

int sbg_batch_device_bytes(sbg_batch b, int64_t* bytes) {
    if (!b || !bytes) return fail(SBG_ERR_INVALID, "null argument");
    *bytes = b->devBytes;
    return SBG_OK;
}

void* sbg_batch_stream(sbg_batch b) { return b ? (void*)b->stream : nullptr; }
int64_t sbg_batch_launch_count(sbg_batch b) { return b ? b->launches : 0; }

int sbg_batch_set_state(sbg_batch b, const double* t, const double* y) {
    if (!b || !y) return fail(SBG_ERR_INVALID, "null argument");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    const size_t bytes = b->nyTotal * sizeof(double);
    const double* src = y;
    if (!isPinned(y)) {
        std::memcpy(b->hostPinned, y, bytes);
        src = b->hostPinned;
    }
    SBG_CUDA(cudaMemcpyAsync(b->staging, src, bytes, cudaMemcpyHostToDevice, b->stream), "state upload");
    SBG_CUDA(launchScatter(b->T, b->dHostYOff, b->staging, b->y, 0, b->stream), "state scatter");
    ++b->launches;
    if (t) {
        SBG_CUDA(cudaStreamSynchronize(b->stream), "state upload");
        std::memcpy(b->hostPinned, t, b->ninst * sizeof(double));
        SBG_CUDA(cudaMemcpyAsync(b->time, b->hostPinned, b->ninst * sizeof(double), cudaMemcpyHostToDevice, b->stream),
                 "time upload");
    } else {
        SBG_CUDA(cudaMemsetAsync(b->time, 0, std::max(b->ninst, 1) * sizeof(double), b->stream), "time reset");
    }
    SBG_CUDA(cudaStreamSynchronize(b->stream), "state upload");
    b->stateSet = true;
    b->integrating = false;
    b->realized = false;
    return SBG_OK;
}

int sbg_batch_get_state(sbg_batch b, double* t, double* y) {
    if (!b || !y) return fail(SBG_ERR_INVALID, "null argument");
    if (!b->stateSet) return fail(SBG_ERR_STATE, "no state has been set");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    SBG_CUDA(launchGather(b->T, b->dHostYOff, b->y, b->staging, 0, b->stream), "state gather");
    ++b->launches;
    double* dst = isPinned(y) ? y : b->hostPinned;
    SBG_CUDA(cudaMemcpyAsync(dst, b->staging, b->nyTotal * sizeof(double), cudaMemcpyDeviceToHost, b->stream),
             "state download");
    SBG_CUDA(cudaStreamSynchronize(b->stream), "state download");
    if (dst != y) std::memcpy(y, b->hostPinned, b->nyTotal * sizeof(double));
    if (t) SBG_CUDA(cudaMemcpy(t, b->time, b->ninst * sizeof(double), cudaMemcpyDeviceToHost), "time download");
    return SBG_OK;
}

// Tuner: the FP32 kernels come in two register budgets (all the registers
// they want, 2 blocks of 128 threads per SM; or at most 128, 4 blocks per SM
// with a few spills), and the level-parallel segment can give each tree more
// or fewer lanes (G = pow2ceil(widest level) >> shift). The first realize or
// integration of a batch times the candidates on the batch's own state and
// keeps the fastest (the realize leaves the state untouched).
static int timePlan(sbg_batch b, float* ms) {
    for (int rep = 0; rep < 2; ++rep)
        SBG_CUDA(launchRealize(b->T, b->plan(), b->precision, b->y, b->ydot, b->bufsArg(), b->status, b->streams()),
                 "tuner launch");
    SBG_CUDA(cudaEventRecord(b->evT0, b->stream), "tuner");
    for (int rep = 0; rep < 3; ++rep)
        SBG_CUDA(launchRealize(b->T, b->plan(), b->precision, b->y, b->ydot, b->bufsArg(), b->status, b->streams()),
                 "tuner launch");
    SBG_CUDA(cudaEventRecord(b->evT1, b->stream), "tuner");
    SBG_CUDA(cudaEventSynchronize(b->evT1), "tuner");
    SBG_CUDA(cudaEventElapsedTime(ms, b->evT0, b->evT1), "tuner");
    b->launches += 5 * b->realizeLaunches();
    return SBG_OK;
}

static int tuneVariant(sbg_batch b) {
    if (b->tuned) return SBG_OK;
    if (!b->evT0) {
        SBG_CUDA(cudaEventCreate(&b->evT0), "tuner");
        SBG_CUDA(cudaEventCreate(&b->evT1), "tuner");
    }
    const bool fixedVariant = b->variant != 0;
    if (!fixedVariant) b->variant = 1;
    float best = 1e30f, ms = 0;
    int bestShift = b->groupShift;
    if (!b->groupWidthKey.empty()) {
        for (int shift : {0, 1, 2}) {
            if (int rc = b->setGroupShift(shift)) return rc;
            if (int rc = timePlan(b, &ms)) return rc;
            if (ms < best) { best = ms; bestShift = shift; }
        }
        if (int rc = b->setGroupShift(bestShift)) return rc;
    } else if (int rc = timePlan(b, &best)) {
        return rc;
    }
    if (!fixedVariant && b->precision != SBG_PRECISION_FP64) {
        int bestVariant = 1;
        for (int v : {4, 7, 8}) {
            if (v >= 7 && b->nChain == 0) continue;  // 64-thread blocks exist for the chain driver only
            if (v == 8 && !b->stagedOk) continue;
            b->variant = v;
            if (int rc = timePlan(b, &ms)) return rc;
            if (ms < best) { best = ms; bestVariant = v; }
        }
        b->variant = bestVariant;
    }
    b->tuned = true;
    return SBG_OK;
}

int sbg_batch_kernel_variant(sbg_batch b) { return b ? (b->tuned ? b->variant : 0) : -1; }
int sbg_batch_group_lanes_shift(sbg_batch b) { return b ? b->groupShift : -1; }

int sbg_realize_acceleration_async(sbg_batch b) {
    if (!b) return fail(SBG_ERR_INVALID, "null batch");
    if (!b->stateSet) return fail(SBG_ERR_STATE, "no state has been set");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    if (int rc = tuneVariant(b)) return rc;
    // The tuned launch sequence (chain segment on the main stream, tree
    // segment forked onto the side stream) is captured once as a CUDA graph
    // and replayed.
    if (!b->realizeGraph) {
        cudaGraph_t g = nullptr;
        SBG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
        cudaError_t e = launchRealize(b->T, b->plan(), b->precision, b->y, b->ydot, b->bufsArg(), b->status, b->streams());
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) return cudaFail(e, "realize capture");
        if (e2 != cudaSuccess) return cudaFail(e2, "graph capture");
        e = cudaGraphInstantiate(&b->realizeGraph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cudaFail(e, "graph instantiate");
    }
    SBG_CUDA(cudaGraphLaunch(b->realizeGraph, b->stream), "realize graph launch");
    b->launches += b->realizeLaunches();
    b->realized = true;
    return SBG_OK;
}

int sbg_batch_get_ydot(sbg_batch b, double* ydot, int32_t* status) {
    if (!b) return fail(SBG_ERR_INVALID, "null batch");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    double* dst = ydot && isPinned(ydot) ? ydot : b->hostPinned;
    if (ydot) {
        SBG_CUDA(launchGather(b->T, b->dHostYOff, b->ydot, b->staging, 0, b->stream), "derivative gather");
        ++b->launches;
        SBG_CUDA(cudaMemcpyAsync(dst, b->staging, b->nyTotal * sizeof(double), cudaMemcpyDeviceToHost, b->stream),
                 "derivative download");
    }
    if (status)
        SBG_CUDA(cudaMemcpyAsync(status, b->status, b->ninst * sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream),
                 "status download");
    SBG_CUDA(cudaStreamSynchronize(b->stream), "derivative download");
    if (ydot && dst != ydot) std::memcpy(ydot, b->hostPinned, b->nyTotal * sizeof(double));
    return SBG_OK;
}

int sbg_realize_acceleration(sbg_batch b, double* ydot, int32_t* status) {
    int rc = sbg_realize_acceleration_async(b);
    if (rc) return rc;
    return sbg_batch_get_ydot(b, ydot, status);
}

// State::updY + realize(Stage::Acceleration) + getYDot from and to host
// buffers in one call. For a batch whose instances all run the one-thread
// driver in instance order, the instances are cut into tile-aligned chunks:
// one stream uploads the chunks in order, three streams scatter, realize and
// gather them as their uploads land, and one stream downloads them in order
// as they finish. The copies of one direction thus go one chunk at a time at
// the link's full rate (concurrent copies would share it, so that the first
// chunk would arrive no sooner than the last), and a chunk's compute overlaps
// the other chunks' copies. Other batches take the plain sequence.
int sbg_realize_acceleration_host(sbg_batch b, const double* y, double* ydot, int32_t* status) {
    if (!b || !y || !ydot) return fail(SBG_ERR_INVALID, "null argument");
    int nchunks = 4;
    if (const char* v = std::getenv("SBG_PIPE_CHUNKS")) nchunks = std::max(1, std::atoi(v));  // tuning override
    nchunks = std::min(nchunks, 16);
    const bool pipelined = b->orderIdentity && b->nGroupBlocks == 0 && b->nLoop == 0 && b->tuned && nchunks > 1 &&
                           b->ninst >= nchunks * kTile;
    if (!pipelined) {
        if (int rc = sbg_batch_set_state(b, nullptr, y)) return rc;
        return sbg_realize_acceleration(b, ydot, status);
    }
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    const size_t bytes = b->nyTotal * sizeof(double);
    const double* src = y;
    if (!isPinned(y)) {
        std::memcpy(b->hostPinned, y, bytes);
        src = b->hostPinned;
    }
    const bool dstPinned = isPinned(ydot);
    double* dst = dstPinned ? ydot : b->hostPinned;
    const bool stPinned = status && isPinned(status);
    b->pipe[0] = b->stream;
    for (int k = 1; k < 5; ++k)
        if (!b->pipe[k]) SBG_CUDA(cudaStreamCreateWithFlags(&b->pipe[k], cudaStreamNonBlocking), "streams");
    for (auto& row : b->pipeEv)
        for (cudaEvent_t& e : row)
            if (!e) SBG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "events");
    if (!b->pipeStart) {
        SBG_CUDA(cudaEventCreateWithFlags(&b->pipeStart, cudaEventDisableTiming), "events");
        SBG_CUDA(cudaEventCreateWithFlags(&b->pipeEnd, cudaEventDisableTiming), "events");
    }
    cudaStream_t up = b->pipe[0], down = b->pipe[4];
    SBG_CUDA(cudaMemsetAsync(b->time, 0, std::max(b->ninst, 1) * sizeof(double), up), "time reset");
    // every stream starts after the work already queued on the batch stream
    SBG_CUDA(cudaEventRecord(b->pipeStart, up), "pipeline");
    for (int k = 1; k < 5; ++k) SBG_CUDA(cudaStreamWaitEvent(b->pipe[k], b->pipeStart, 0), "pipeline");
    const int tiles = (b->ninst + kTile - 1) / kTile;
    KArgs a{};
    a.T = &b->T;
    a.y = b->y;
    a.ydot = b->ydot;
    a.scratch = b->scratch;
    a.status = b->status;
    for (int c = 0; c < nchunks; ++c) {
        const int i0 = std::min(b->ninst, (int)((int64_t)tiles * c / nchunks) * kTile);
        const int i1 = std::min(b->ninst, (int)((int64_t)tiles * (c + 1) / nchunks) * kTile);
        if (i1 <= i0) continue;
        const int64_t o0 = b->hostYOff[i0], o1 = b->hostYOff[i1];
        cudaStream_t st = b->pipe[1 + c % 3];
        SBG_CUDA(cudaMemcpyAsync(b->staging + o0, src + o0, (o1 - o0) * sizeof(double), cudaMemcpyHostToDevice, up),
                 "state upload");
        SBG_CUDA(cudaEventRecord(b->pipeEv[0][c], up), "pipeline");
        SBG_CUDA(cudaStreamWaitEvent(st, b->pipeEv[0][c], 0), "pipeline");
        SBG_CUDA(launchScatter(b->T, b->dHostYOff, b->staging, b->y, 0, st, i0, i1 - i0), "state scatter");
        LaunchPlan P = b->plan();
        P.chainFirst = i0;
        P.nChain = i1 - i0;
        a.P = &P;
        if (b->precision == SBG_PRECISION_FP64) realize64Chain(a, st);
        else realize32Chain(a, b->precision == SBG_PRECISION_MIXED, st);
        SBG_CUDA(cudaGetLastError(), "realize launch");
        SBG_CUDA(launchGather(b->T, b->dHostYOff, b->ydot, b->staging, 0, st, i0, i1 - i0), "derivative gather");
        SBG_CUDA(cudaEventRecord(b->pipeEv[1][c], st), "pipeline");
        SBG_CUDA(cudaStreamWaitEvent(down, b->pipeEv[1][c], 0), "pipeline");
        SBG_CUDA(cudaMemcpyAsync(dst + o0, b->staging + o0, (o1 - o0) * sizeof(double), cudaMemcpyDeviceToHost, down),
                 "derivative download");
        if (stPinned)
            SBG_CUDA(cudaMemcpyAsync(status + i0, b->status + i0, (i1 - i0) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                     down), "status download");
        b->launches += 3 + (b->T.scratch64 ? 1 : 0);
    }
    if (status && !stPinned)
        SBG_CUDA(cudaMemcpyAsync(status, b->status, b->ninst * sizeof(int32_t), cudaMemcpyDeviceToHost, down),
                 "status download");
    // the batch stream continues after the downloads
    SBG_CUDA(cudaEventRecord(b->pipeEnd, down), "pipeline");
    SBG_CUDA(cudaStreamWaitEvent(b->stream, b->pipeEnd, 0), "pipeline");
    SBG_CUDA(cudaStreamSynchronize(down), "pipelined realize");
    if (!dstPinned) std::memcpy(ydot, b->hostPinned, bytes);
    b->stateSet = true;
    b->integrating = false;
    b->realized = true;
    return SBG_OK;
}

int sbg_multiply_by_minv(sbg_batch b, const double* f, double* outp) {
    if (!b || !f || !outp) return fail(SBG_ERR_INVALID, "null argument");
    if (!b->stateSet) return fail(SBG_ERR_STATE, "no state has been set");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    const size_t bytes = b->nuTotal * sizeof(double);
    std::memcpy(b->hostPinned, f, bytes);
    SBG_CUDA(cudaMemcpyAsync(b->staging, b->hostPinned, bytes, cudaMemcpyHostToDevice, b->stream), "force upload");
    SBG_CUDA(launchScatter(b->T, b->dHostUOff, b->staging, b->fcol, 1, b->stream), "force scatter");
    SBG_CUDA(launchMInv(b->T, b->plan(), b->precision, b->y, b->fcol, b->ydot, b->bufsArg(), b->status, b->streams()),
             "M^-1 kernel launch");
    b->realized = false;  // the result went to the derivative columns
    SBG_CUDA(launchGather(b->T, b->dHostUOff, b->ydot, b->staging, 1, b->stream), "result gather");
    b->launches += 2 + b->segments();
    SBG_CUDA(cudaMemcpyAsync(b->hostPinned, b->staging, bytes, cudaMemcpyDeviceToHost, b->stream), "result download");
    SBG_CUDA(cudaStreamSynchronize(b->stream), "M^-1");
    std::memcpy(outp, b->hostPinned, bytes);
    return SBG_OK;
}

// ------------------------------------------------------------ tree operators
// Device operands of a tree operator in the host packing: x [nu] | fmob [nu] |
// fbody [6 nb] | out [max(nu, 10 nb)], mirrored in pinned host memory.
static int ensureTreeOps(sbg_batch b) {
    const int64_t nu = b->nuTotal, nbT = b->hostBOff[b->ninst];
    const int64_t need = 2 * nu + 6 * nbT + std::max<int64_t>(nu, 10 * nbT);
    if (b->opsDev && b->opsElems >= need) return SBG_OK;
    int rc;
    void* p = nullptr;
    if (b->precision != SBG_PRECISION_FP64 && !b->opsScratch && b->scratchElems > 0) {
        if (b->T.scratch64) b->opsScratch = b->T.scratch64;  // the mixed form's FP64 mirror has the layout
        else if ((rc = b->alloc(&b->opsScratch, b->scratchElems * sizeof(double), "tree-operator scratch"))) return rc;
    }
    if ((rc = b->alloc(&p, std::max<int64_t>(need, 1) * sizeof(double), "tree-operator operands"))) return rc;
    b->opsDev = static_cast<double*>(p);
    const int64_t* dOff = nullptr;
    if ((rc = b->upload(&dOff, b->hostBOff, "offsets"))) return rc;
    b->dHostBOff = const_cast<int64_t*>(dOff);
    cudaError_t e = cudaMallocHost(&b->opsHost, std::max<int64_t>(need, 1) * sizeof(double));
    if (e != cudaSuccess) {
        b->opsHost = nullptr;
        return cudaFail(e, "cudaMallocHost");
    }
    b->opsElems = need;
    if (!b->evOp0) {
        SBG_CUDA(cudaEventCreate(&b->evOp0), "event");
        SBG_CUDA(cudaEventCreate(&b->evOp1), "event");
    }
    return SBG_OK;
}

static int runTreeOp(sbg_batch b, int kind, const double* x, const double* fmob, const double* fbody, double* out,
                     int32_t* status) {
    if (!b || !out) return fail(SBG_ERR_INVALID, "null argument");
    if (!b->stateSet) return fail(SBG_ERR_STATE, "no state has been set");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    if (int rc = ensureTreeOps(b)) return rc;
    const int64_t nu = b->nuTotal, nbT = b->hostBOff[b->ninst];
    double* dX = b->opsDev;
    double* dF = dX + nu;
    double* dB = dF + nu;
    double* dOut = dB + 6 * nbT;
    const int64_t nOut = kind == OP_JV ? 6 * nbT : (kind == OP_COMPOSITE ? 10 * nbT : nu);
    double* hX = b->opsHost;
    auto up = [&](const double* src, double* dDst, int64_t n, const char* what) -> int {
        if (!src || n == 0) return SBG_OK;
        double* h = hX + (dDst - b->opsDev);
        std::memcpy(h, src, n * sizeof(double));
        SBG_CUDA(cudaMemcpyAsync(dDst, h, n * sizeof(double), cudaMemcpyHostToDevice, b->stream), what);
        return SBG_OK;
    };
    if (int rc = up(x, dX, nu, "operand upload")) return rc;
    if (int rc = up(fmob, dF, nu, "mobility force upload")) return rc;
    if (int rc = up(fbody, dB, 6 * nbT, "body force upload")) return rc;
    OpIO io{kind, x ? dX : nullptr, fmob ? dF : nullptr, fbody ? dB : nullptr, dOut, b->dHostUOff, b->dHostBOff};
    double* sc = b->precision == SBG_PRECISION_FP64 ? static_cast<double*>(b->scratch)
                                                     : static_cast<double*>(b->opsScratch);
    SBG_CUDA(cudaEventRecord(b->evOp0, b->stream), "event");
    SBG_CUDA(launchTreeOp(b->T, b->plan(), io, b->y, sc, static_cast<double*>(b->scratchLoop), b->status, b->stream),
             "tree-operator kernel launch");
    SBG_CUDA(cudaEventRecord(b->evOp1, b->stream), "event");
    b->launches += b->segments();
    double* hOut = hX + (dOut - b->opsDev);
    if (nOut > 0)
        SBG_CUDA(cudaMemcpyAsync(hOut, dOut, nOut * sizeof(double), cudaMemcpyDeviceToHost, b->stream), "result download");
    if (status && b->ninst > 0)
        SBG_CUDA(cudaMemcpyAsync(status, b->status, b->ninst * sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream),
                 "status download");
    SBG_CUDA(cudaStreamSynchronize(b->stream), "tree operator");
    std::memcpy(out, hOut, nOut * sizeof(double));
    return SBG_OK;
}

int sbg_batch_fallback_count(sbg_batch b, int64_t* n) {
    if (!b || !n) return fail(SBG_ERR_INVALID, "null argument");
    *n = 0;
    if (!b->T.fallbacks) return SBG_OK;
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    unsigned long long v = 0;
    SBG_CUDA(cudaStreamSynchronize(b->stream), "fallback count");
    SBG_CUDA(cudaMemcpy(&v, b->T.fallbacks, sizeof(v), cudaMemcpyDeviceToHost), "fallback count");
    *n = (int64_t)v;
    return SBG_OK;
}

int sbg_batch_fp64_steps(sbg_batch b, int64_t* n) {
    if (!b || !n) return fail(SBG_ERR_INVALID, "null argument");
    *n = 0;
    if (!b->fbSteps) return SBG_OK;
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    unsigned long long v = 0;
    SBG_CUDA(cudaStreamSynchronize(b->stream), "FP64 step count");
    SBG_CUDA(cudaMemcpy(&v, b->fbSteps, sizeof(v), cudaMemcpyDeviceToHost), "FP64 step count");
    *n = (int64_t)v;
    return SBG_OK;
}

int sbg_batch_last_operator_ms(sbg_batch b, double* ms) {
    if (!b || !ms) return fail(SBG_ERR_INVALID, "null argument");
    if (!b->evOp0) return fail(SBG_ERR_STATE, "no tree operator has run");
    float t = 0.f;
    SBG_CUDA(cudaEventElapsedTime(&t, b->evOp0, b->evOp1), "event");
    *ms = t;
    return SBG_OK;
}

int sbg_calc_residual_force(sbg_batch b, const double* mobility_forces, const double* body_forces,
                            const double* known_udot, double* residual, int32_t* status) {
    return runTreeOp(b, OP_RESIDUAL, known_udot, mobility_forces, body_forces, residual, status);
}
int sbg_multiply_by_m(sbg_batch b, const double* a, double* Ma, int32_t* status) {
    if (!a) return fail(SBG_ERR_INVALID, "null argument");
    return runTreeOp(b, OP_MV, a, nullptr, nullptr, Ma, status);
}
int sbg_multiply_by_system_jacobian(sbg_batch b, const double* u, double* Ju, int32_t* status) {
    if (!u) return fail(SBG_ERR_INVALID, "null argument");
    return runTreeOp(b, OP_JV, u, nullptr, nullptr, Ju, status);
}
int sbg_multiply_by_system_jacobian_transpose(sbg_batch b, const double* F_G, double* f, int32_t* status) {
    if (!F_G) return fail(SBG_ERR_INVALID, "null argument");
    return runTreeOp(b, OP_JTF, nullptr, nullptr, F_G, f, status);
}
int sbg_calc_composite_body_inertias(sbg_batch b, double* R, int32_t* status) {
    return runTreeOp(b, OP_COMPOSITE, nullptr, nullptr, nullptr, R, status);
}

// The number of steps takeOneStep's rule takes from t0 to tStop with step h
// (AbstractIntegratorRep.cpp:536-544), as the RK kernels apply it.
static int64_t stepsToReach(double t0, double tStop, double h) {
    int64_t n = 0;
    double tc = t0;
    while (tc < tStop && n < kMaxStepsPerCall) {
        double t1;
        if (tStop < tc + 0.95 * h) t1 = tStop;
        else if (tStop > tc + 1.001 * h) t1 = tc + h;
        else t1 = tStop;
        if (!(t1 > tc)) break;
        tc = t1;
        ++n;
    }
    return n;
}

// Buffers of the one-step launches of a mixed batch integration (allocated
// on first use): the two FP64-mode lists and their lengths, the per-instance
// FP64 modes and step counters, the FP64 stage planes, FP64 records of the
// level-parallel layout for the list kernel, its stream and events.
static int ensureFallbackSteps(sbg_batch b) {
    if (b->fbList) return SBG_OK;
    void* p = nullptr;
    int rc;
    const int64_t n = b->ninst;
    if ((rc = b->alloc(&p, 2 * n * sizeof(int32_t), "FP64 lists"))) return rc;
    b->fbList = static_cast<int32_t*>(p);
    if ((rc = b->alloc(&p, 4 * sizeof(int32_t), "FP64 list lengths"))) return rc;
    b->fbCount = static_cast<int32_t*>(p);
    if ((rc = b->alloc(&p, 2 * n * sizeof(int32_t), "FP64 modes"))) return rc;
    b->fbMode = static_cast<int32_t*>(p);
    if ((rc = b->alloc(&p, n * sizeof(int32_t), "FP64 step counters"))) return rc;
    b->fbLeft = static_cast<int32_t*>(p);
    if ((rc = b->alloc(&p, n * sizeof(int32_t), "step counters"))) return rc;
    b->stepsLeft = static_cast<int32_t*>(p);
    if ((rc = b->alloc(&p, 4 * std::max<int64_t>(b->colElems, 1) * sizeof(double), "FP64 stage derivatives")))
        return rc;
    b->fbuf64 = static_cast<double*>(p);
    if ((rc = b->alloc(&p, sizeof(unsigned long long), "FP64 step counter"))) return rc;
    b->fbSteps = static_cast<unsigned long long*>(p);
    SBG_CUDA(cudaMemsetAsync(b->fbSteps, 0, sizeof(unsigned long long), b->stream), "FP64 step counter");
    std::vector<int64_t> base(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) base[i + 1] = base[i] + b->rowsElems[i];
    if ((rc = b->alloc(&p, std::max<int64_t>(base[n], 1) * sizeof(double), "FP64 level-parallel records"))) return rc;
    b->rows = static_cast<double*>(p);
    const int64_t* dBase = nullptr;
    if ((rc = b->upload(&dBase, base, "FP64 record offsets"))) return rc;
    b->rowsBase = const_cast<int64_t*>(dBase);
    SBG_CUDA(cudaStreamCreateWithFlags(&b->fbStream, cudaStreamNonBlocking), "stream");
    SBG_CUDA(cudaEventCreateWithFlags(&b->fbFork, cudaEventDisableTiming), "event");
    SBG_CUDA(cudaEventCreateWithFlags(&b->fbJoin, cudaEventDisableTiming), "event");
    return SBG_OK;
}

// Launches per window of the FP64 share test of a mixed batch integration.
constexpr int64_t kFp64Window = 64;

// A mixed batch integration as one-step launches. At launch L the mixed
// kernels step the instances in mixed mode while the FP64 list kernel, on its
// own stream, steps those in FP64 mode; an instance whose mixed step meets an
// ill-conditioned M keeps its state and takes that step in FP64 at launch
// L + 1, so it ends one launch behind the others for each such event.
// Launches go on until every instance has taken its steps (nsteps >= 0) or
// reached tStop. Every kFp64Window launches the share of instance steps taken
// in FP64 is checked; above a quarter, the integration switches for good (its
// continued calls too) to the FP64 persistent kernels: on chaotic trees the
// mixed steps then save less than the FP64 ones cost beside them.
static int rkMersonMixedSteps(sbg_batch b, double h, int32_t nsteps, double tStop, bool cont, double acc, double ctol,
                              int pes) {
    if (int rc = ensureFallbackSteps(b)) return rc;
    DevTables Tk = b->T;
    Tk.fbList = b->fbList;
    Tk.fbCount = b->fbCount;
    Tk.fbMode = b->fbMode;
    Tk.fbLeft = b->fbLeft;
    Tk.stepsLeft = nsteps >= 0 ? b->stepsLeft : nullptr;
    Tk.fbuf64 = b->fbuf64;
    Tk.fbSteps = b->fbSteps;
    const int n = b->ninst;
    if (!cont) {  // a new integration: every instance starts in mixed mode
        SBG_CUDA(cudaMemsetAsync(b->fbMode, 0, 2 * (size_t)n * sizeof(int32_t), b->stream), "FP64 modes");
        SBG_CUDA(cudaMemsetAsync(b->fbLeft, 0, n * sizeof(int32_t), b->stream), "FP64 modes");
        SBG_CUDA(cudaMemsetAsync(b->fbCount, 0, 2 * sizeof(int32_t), b->stream), "FP64 lists");
        b->fbLaunch = 0;
        b->fbAllFp64 = false;
        b->fbWindow0 = 0;
        SBG_CUDA(cudaStreamSynchronize(b->stream), "FP64 step count");
        SBG_CUDA(cudaMemcpy(&b->fbWindow0, b->fbSteps, sizeof(unsigned long long), cudaMemcpyDeviceToHost),
                 "FP64 step count");
    }
    int64_t target = nsteps;
    if (nsteps >= 0) {
        SBG_CUDA(launchFillInt(b->stepsLeft, n, nsteps, b->stream), "step counters");
    } else {
        // steps to tStop from the earliest instance time, by the kernels' rule
        std::vector<double> t0(n);
        SBG_CUDA(cudaMemcpyAsync(t0.data(), b->time, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream),
                 "time download");
        SBG_CUDA(cudaStreamSynchronize(b->stream), "time download");
        target = stepsToReach(*std::min_element(t0.begin(), t0.end()), tStop, h);
    }
    const LaunchPlan P = b->plan();
    // FP64 steps: kFbLanes level-parallel lanes per instance (measured faster
    // than one thread per instance: 2.4x on the uneven trees, 6 % on the
    // random trees)
    int fbLanes = kFbLanes;
    if (const char* v = std::getenv("SBG_FB_LANES")) fbLanes = std::atoi(v) > 1 ? kFbLanes : 1;  // tuning override
    const int64_t limit = 2 * target + 64;
    // The FP64 persistent kernels, on the FP64 mirror of the records, take
    // every instance's remaining steps once the integration has switched.
    auto allFp64 = [&]() -> int {
        const BatchBufs B64{b->T.scratch64, b->scratchLoop, b->fbuf64, b->fbufLoop ? b->fbufLoop : b->fbuf64,
                            b->colElems};
        const StepCtl step{nsteps >= 0 ? nsteps : -1, 0, tStop, 0, 0};
        SBG_CUDA(launchRKMerson(Tk, P, SBG_PRECISION_FP64, b->y, b->time, B64, b->status, h, step, acc, ctol, pes,
                                b->streams()),
                 "RK-Merson kernel launch");
        b->launches += b->segments();
        return SBG_OK;
    };
    if (b->fbAllFp64) return allFp64();
    int64_t L = 0;
    for (;;) {
        for (; L < target; ++L) {
            const int64_t G = b->fbLaunch + L;  // launch index within the whole integration
            if (G > 0 && G % kFp64Window == 0) {
                // more than a quarter of the last window's instance steps in FP64:
                // the FP64 kernels take the rest, without the mixed steps' overhead
                unsigned long long v = 0;
                SBG_CUDA(cudaStreamSynchronize(b->stream), "FP64 step count");
                SBG_CUDA(cudaMemcpy(&v, b->fbSteps, sizeof(v), cudaMemcpyDeviceToHost), "FP64 step count");
                const unsigned long long d = v - b->fbWindow0;
                b->fbWindow0 = v;
                if (4 * d > (unsigned long long)n * kFp64Window) {
                    b->fbAllFp64 = true;
                    b->fbLaunch += L;
                    return allFp64();
                }
            }
            const int li = (int)(G & ((1 << 30) - 1));  // only its parity matters
            SBG_CUDA(cudaMemsetAsync(b->fbCount + ((li + 1) & 1), 0, sizeof(int32_t), b->stream), "FP64 list reset");
            SBG_CUDA(cudaEventRecord(b->fbFork, b->stream), "fork");
            SBG_CUDA(cudaStreamWaitEvent(b->fbStream, b->fbFork, 0), "fork");
            const StepCtl step{nsteps >= 0 ? 1 : -1, (!cont && L == 0) ? 1 : 0, tStop, 1, li};
            SBG_CUDA(launchRKMerson(Tk, P, b->precision, b->y, b->time, b->bufsArg(), b->status, h, step, acc, ctol, pes,
                                    b->streams()),
                     "RK-Merson kernel launch");
            SBG_CUDA(launchRKFp64List(Tk, P, b->y, b->time, b->status, h, step, acc, ctol, pes, b->colElems, b->rowsBase,
                                      b->rows, fbLanes, b->fbStream),
                     "FP64 list kernel launch");
            SBG_CUDA(cudaEventRecord(b->fbJoin, b->fbStream), "join");
            SBG_CUDA(cudaStreamWaitEvent(b->stream, b->fbJoin, 0), "join");
            b->launches += b->segments() + 1;
        }
        SBG_CUDA(launchCountUnfinished(n, Tk.stepsLeft, b->time, b->status, tStop, b->fbCount + 2, b->stream),
                 "unfinished count");
        int32_t left = 0;
        SBG_CUDA(cudaMemcpyAsync(&left, b->fbCount + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream),
                 "unfinished count");
        SBG_CUDA(cudaStreamSynchronize(b->stream), "unfinished count");
        if (left == 0) break;
        if (L >= limit) return fail(SBG_ERR_CUDA, "mixed integration did not finish its steps");
        target = L + 4;
    }
    b->fbLaunch += L;
    return SBG_OK;
}

// One integration call: Integrator::initialize (unless the options continue
// the previous call's integration), then the steps StepCtl describes.
static int rkMersonCall(sbg_batch b, double h, int32_t nsteps, double tStop, const sbg_integ_opts* opts) {
    if (!b) return fail(SBG_ERR_INVALID, "null batch");
    if (!b->stateSet) return fail(SBG_ERR_STATE, "no state has been set");
    if (!(h > 0) || !std::isfinite(h)) return fail(SBG_ERR_INVALID, "step size must be positive");
    if (nsteps < 0 && !std::isfinite(tStop)) return fail(SBG_ERR_INVALID, "report time must be finite");
    double acc = 1e-3, ctol = -1;
    int pes = 0;
    bool cont = false;
    if (opts) {
        if (opts->accuracy > 0) acc = opts->accuracy;
        if (opts->constraint_tolerance > 0) ctol = opts->constraint_tolerance;
        pes = opts->project_every_step;
        cont = opts->continue_integration != 0;
    }
    if (ctol <= 0) ctol = acc / 10;
    if (cont && !b->integrating)
        return fail(SBG_ERR_STATE, "no integration to continue: the state was set since, or none has run");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    if (int rc = tuneVariant(b)) return rc;  // realize leaves the state untouched
    SBG_CUDA(cudaMemsetAsync(b->status, 0, std::max(b->ninst, 1) * sizeof(int32_t), b->stream), "status reset");
    if (!cont) {
        SBG_CUDA(launchNormalizeQuat(b->T, b->y, b->stream), "initialize");
        ++b->launches;
    }
    if (b->precision == SBG_PRECISION_MIXED && b->ninst > 0) {
        // one step per launch: steps that meet an ill-conditioned M are taken in FP64
        if (int rc = rkMersonMixedSteps(b, h, nsteps, tStop, cont, acc, ctol, pes)) return rc;
    } else {
        const StepCtl step{nsteps, cont ? 0 : 1, tStop, 0, 0};
        SBG_CUDA(launchRKMerson(b->T, b->plan(), b->precision, b->y, b->time, b->bufsArg(), b->status, h, step, acc,
                                ctol, pes, b->streams()),
                 "RK-Merson kernel launch");
        b->launches += b->segments();
    }
    b->integrating = true;
    b->realized = false;
    return SBG_OK;
}

static int rkMersonFinish(sbg_batch b, int32_t* status) {
    SBG_CUDA(cudaStreamSynchronize(b->stream), "RK-Merson");
    if (status) SBG_CUDA(cudaMemcpy(status, b->status, b->ninst * sizeof(int32_t), cudaMemcpyDeviceToHost), "status download");
    return SBG_OK;
}

int sbg_rk_merson_fixed_async(sbg_batch b, double h, int32_t nsteps, const sbg_integ_opts* opts) {
    if (nsteps < 0) return fail(SBG_ERR_INVALID, "negative step count");
    return rkMersonCall(b, h, nsteps, 0.0, opts);
}

int sbg_rk_merson_fixed(sbg_batch b, double h, int32_t nsteps, const sbg_integ_opts* opts, int32_t* status) {
    int rc = sbg_rk_merson_fixed_async(b, h, nsteps, opts);
    if (rc) return rc;
    return rkMersonFinish(b, status);
}

int sbg_rk_merson_step_to_async(sbg_batch b, double h, double t_report, const sbg_integ_opts* opts) {
    return rkMersonCall(b, h, -1, t_report, opts);
}

int sbg_rk_merson_step_to(sbg_batch b, double h, double t_report, const sbg_integ_opts* opts, int32_t* status) {
    int rc = sbg_rk_merson_step_to_async(b, h, t_report, opts);
    if (rc) return rc;
    return rkMersonFinish(b, status);
}

int sbg_batch_get_qdotdot(sbg_batch b, double* qdotdot) {
    if (!b || !qdotdot) return fail(SBG_ERR_INVALID, "null argument");
    if (!b->realized) return fail(SBG_ERR_STATE, "the current state has not been realized through Acceleration");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    const int64_t nqT = b->nyTotal - b->nuTotal;
    SBG_CUDA(launchQDotDot(b->T, b->dHostQOff, b->y, b->ydot, b->staging, b->stream), "qdotdot kernel launch");
    ++b->launches;
    SBG_CUDA(cudaMemcpyAsync(b->hostPinned, b->staging, nqT * sizeof(double), cudaMemcpyDeviceToHost, b->stream),
             "qdotdot download");
    SBG_CUDA(cudaStreamSynchronize(b->stream), "qdotdot");
    std::memcpy(qdotdot, b->hostPinned, nqT * sizeof(double));
    return SBG_OK;
}

int sbg_rk_merson_adaptive(sbg_batch b, double t_final, const sbg_adaptive_opts* opts, int32_t* status,
                           int64_t* stats) {
    if (!b) return fail(SBG_ERR_INVALID, "null batch");
    if (!b->stateSet) return fail(SBG_ERR_STATE, "no state has been set");
    if (!std::isfinite(t_final)) return fail(SBG_ERR_INVALID, "final time must be finite");
    if (b->precision != SBG_PRECISION_FP64)
        return fail(SBG_ERR_UNSUPPORTED, "the error-controlled integrator runs on FP64 batches");
    if (b->nLoop > 0) return fail(SBG_ERR_UNSUPPORTED, "error-controlled integration of loop closures is not supported");
    AdaptCtl ac{};
    ac.tFinal = t_final;
    ac.accuracy = 1e-3;
    ac.consTol = -1;
    ac.maxSteps = 1000000;
    if (opts) {
        if (opts->accuracy > 0) ac.accuracy = opts->accuracy;
        if (opts->constraint_tolerance > 0) ac.consTol = opts->constraint_tolerance;
        ac.hInit = opts->initial_step;
        ac.hMin = opts->min_step;
        ac.hMax = opts->max_step;
        ac.projectEveryStep = opts->project_every_step;
        if (opts->max_steps > 0) ac.maxSteps = opts->max_steps;
    }
    if (ac.consTol <= 0) ac.consTol = ac.accuracy / 10;
    if (ac.hMin > 0 && ac.hMax > 0 && ac.hMin > ac.hMax) return fail(SBG_ERR_INVALID, "minimum step above maximum step");
    SBG_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    if (b->ninst == 0) return SBG_OK;
    if (stats && !b->adaptStats) {
        void* p = nullptr;
        if (int rc = b->alloc(&p, 2 * (size_t)b->ninst * sizeof(long long), "step statistics")) return rc;
        b->adaptStats = static_cast<long long*>(p);
    }
    ac.stats = stats ? b->adaptStats : nullptr;
    SBG_CUDA(cudaMemsetAsync(b->status, 0, b->ninst * sizeof(int32_t), b->stream), "status reset");
    SBG_CUDA(launchNormalizeQuat(b->T, b->y, b->stream), "initialize");  // Integrator::initialize
    KArgs a{};
    const LaunchPlan P = b->plan();
    a.T = &b->T;
    a.P = &P;
    a.ystate = b->y;
    a.time = b->time;
    a.fbuf = b->fbuf;
    a.fplane = b->colElems;
    a.scratch = b->scratch;
    a.status = b->status;
    const Streams ss = b->streams();
    const bool both = P.nChain > 0 && P.nGroupBlocks > 0;
    if (both) {
        SBG_CUDA(cudaEventRecord(ss.fork, ss.main), "fork");
        SBG_CUDA(cudaStreamWaitEvent(ss.side, ss.fork, 0), "fork");
    }
    rkAdaptiveChain(a, ac, ss.main);
    rkAdaptiveGroup(a, ac, both ? ss.side : ss.main);
    SBG_CUDA(cudaGetLastError(), "error-controlled RK-Merson launch");
    if (both) {
        SBG_CUDA(cudaEventRecord(ss.join, ss.side), "join");
        SBG_CUDA(cudaStreamWaitEvent(ss.main, ss.join, 0), "join");
    }
    b->launches += 1 + b->segments();
    b->integrating = false;  // the fixed-step integrator has nothing to continue
    b->realized = false;
    SBG_CUDA(cudaStreamSynchronize(b->stream), "error-controlled RK-Merson");
    if (status) SBG_CUDA(cudaMemcpy(status, b->status, b->ninst * sizeof(int32_t), cudaMemcpyDeviceToHost), "status download");
    if (stats) {
        static_assert(sizeof(long long) == sizeof(int64_t), "statistics are 64-bit");
        SBG_CUDA(cudaMemcpy(stats, b->adaptStats, 2 * (size_t)b->ninst * sizeof(int64_t), cudaMemcpyDeviceToHost),
                 "statistics download");
    }
    return SBG_OK;
}

int sbg_batch_sync(sbg_batch b) {
    if (!b) return fail(SBG_ERR_INVALID, "null batch");
    SBG_CUDA(cudaStreamSynchronize(b->stream), "synchronize");
    return SBG_OK;
}

}  // extern "C"
