// k_noalloc.cu -- realize(Stage::Acceleration) for callers that cannot
// allocate device memory.
//
// Some callers must not call cudaMalloc: a control loop that allocates only at
// start-up, a host framework whose device memory comes from its own pool, or
// code that runs while the allocator is off limits. For them this file holds
// the per-body scratch of the FP64 realize in a file-scope device array, and
// the topology tables in fixed-size device arrays, so one call allocates
// nothing: the caller passes device buffers for the state and the results.
//
// Limits: one topology per call with at most kNoAllocMaxBodies bodies and
// kNoAllocMaxForces mobility-force elements; the scratch array holds
// kNoAllocScratchBytes (16 MiB), enough for 16 MiB / (per-instance record)
// instances at a time -- larger batches are processed in turns by the same
// threads. Every call on every stream shares these arrays: calls that overlap
// on the GPU race and must not be issued concurrently.
#include "abi_device.cuh"
#include "topology_internal.h"

#include <mutex>
#include <string>

namespace sbg {

constexpr int kNoAllocMaxBodies = 256;
constexpr int kNoAllocMaxForces = 4096;
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

// The scratch array. Its host-side name is only a stand-in: kernels get the
// device address obtained with cudaGetSymbolAddress.
static __device__ __align__(256) double g_noallocScratch[kNoAllocScratchBytes / sizeof(double)];

// Topology tables of the current call (one topology, one instance record).
static __device__ __align__(256) int32_t g_naParent[kNoAllocMaxBodies];
static __device__ __align__(256) int32_t g_naInfo[kNoAllocMaxBodies];
static __device__ __align__(256) int32_t g_naQoff[kNoAllocMaxBodies];
static __device__ __align__(256) int32_t g_naUoff[kNoAllocMaxBodies];
static __device__ __align__(256) int32_t g_naSrec[kNoAllocMaxBodies];
static __device__ __align__(256) int32_t g_naFbeg[kNoAllocMaxBodies];
static __device__ __align__(256) int32_t g_naFcnt[kNoAllocMaxBodies];
static __device__ __align__(256) double g_naPar[kNoAllocMaxBodies * kParamStride];
static __device__ __align__(256) int32_t g_naFkw[kNoAllocMaxForces];
static __device__ __align__(256) double g_naFcoef[kNoAllocMaxForces];
static __device__ __align__(256) double g_naFq0[kNoAllocMaxForces];
static __device__ __align__(256) int32_t g_naInst[2];   // first body row, body count
static __device__ __align__(256) double g_naGrav[3];

template <int NM>
__global__ void __launch_bounds__(128) realizeNoAllocKernel(DevTables T, const double* __restrict__ y,
                                                            double* __restrict__ ydot, int32_t* __restrict__ status,
                                                            double* __restrict__ scratch, int ninst, int nq, int ny,
                                                            int64_t recSize) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    const int nthreads = gridDim.x * blockDim.x;
    const ScrRows<double> S{scratch + (int64_t)slot * recSize, 1};  // contiguous record per slot
    for (int inst = slot; inst < ninst; inst += nthreads) {
        const int64_t base = (int64_t)inst * ny;
        YSrc src{y, base, 1, nq};
        YdOut out{ydot, base, 1, nq};
        int st = rhsChain<double, NM, false>(T, 0, S, src, out);
        if (!out.finite) st |= SBG_INST_NONFINITE;
        status[inst] = st;
    }
}

namespace {

thread_local std::string g_naErr;
std::mutex g_naMutex;
double* g_naScratchPtr[64] = {};
DevTables g_naTables[64];
bool g_naReady[64] = {};

template <class T_> cudaError_t symAddr(const T_& sym, const void** p) {
    void* q = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&q, sym);
    *p = q;
    return e;
}

// Once per device, with that device current: device addresses of the arrays.
cudaError_t setUpDevice(int dev) {
    std::lock_guard<std::mutex> lock(g_naMutex);
    if (g_naReady[dev]) return cudaSuccess;
    void* s = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&s, g_noallocScratch);
    if (e != cudaSuccess) return e;
    DevTables T{};
    const void* p = nullptr;
#define SBG_SYM(field, sym, type)                       \
    if ((e = symAddr(sym, &p)) != cudaSuccess) return e; \
    T.field = static_cast<type>(p);
    SBG_SYM(parent, g_naParent, const int32_t*)
    SBG_SYM(info, g_naInfo, const int32_t*)
    SBG_SYM(qoff, g_naQoff, const int32_t*)
    SBG_SYM(uoff, g_naUoff, const int32_t*)
    SBG_SYM(srec, g_naSrec, const int32_t*)
    SBG_SYM(fbeg, g_naFbeg, const int32_t*)
    SBG_SYM(fcnt, g_naFcnt, const int32_t*)
    SBG_SYM(par64, g_naPar, const double*)
    SBG_SYM(fkind_which, g_naFkw, const int32_t*)
    SBG_SYM(fcoef64, g_naFcoef, const double*)
    SBG_SYM(fq064, g_naFq0, const double*)
    SBG_SYM(ibody, g_naInst, const int32_t*)
    SBG_SYM(grav, g_naGrav, const double*)
#undef SBG_SYM
    T.inb = T.ibody + 1;
    T.ninst = 1;
    g_naScratchPtr[dev] = static_cast<double*>(s);
    g_naTables[dev] = T;
    g_naReady[dev] = true;
    return cudaSuccess;
}

int naFail(int code, const std::string& m) {
    g_naErr = m;
    return code;
}

}  // namespace
}  // namespace sbg

using namespace sbg;

extern "C" {

const char* sbg_noalloc_last_error(void) { return g_naErr.c_str(); }

int sbg_realize_acceleration_noalloc(sbg_topology topo, int32_t ninst, const double* y, double* ydot,
                                     int32_t* status, void* stream) {
    if (!topo || ninst < 0 || (ninst > 0 && (!y || !ydot || !status)))
        return naFail(SBG_ERR_INVALID, "null argument or negative instance count");
    if (topo->ncons > 0) return naFail(SBG_ERR_UNSUPPORTED, "loop closures are not supported by the no-alloc path");
    if (topo->ncontacts > 0) return naFail(SBG_ERR_UNSUPPORTED, "contact spheres are not supported by the no-alloc path");
    if (topo->nb > kNoAllocMaxBodies)
        return naFail(SBG_ERR_INVALID, "topology has " + std::to_string(topo->nb) + " bodies; the no-alloc path takes at most " +
                                           std::to_string(kNoAllocMaxBodies));
    if ((int64_t)topo->fkw.size() > kNoAllocMaxForces)
        return naFail(SBG_ERR_INVALID, "topology has " + std::to_string(topo->fkw.size()) +
                                           " mobility forces; the no-alloc path takes at most " +
                                           std::to_string(kNoAllocMaxForces));
    int64_t padRec = 0;
    paddedRecords(*topo, topo->maxNonFreeDof <= 1 ? 1 : 3, &padRec);
    const int64_t recBytes = padRec * (int64_t)sizeof(double);
    if (recBytes > (int64_t)kNoAllocScratchBytes)
        return naFail(SBG_ERR_INVALID, "one instance needs " + std::to_string(recBytes) +
                                           " bytes of scratch, above the no-alloc capacity of " +
                                           std::to_string(kNoAllocScratchBytes) + " bytes");
    if (ninst == 0) return SBG_OK;
    {   // the per-call table uploads read host memory that ends with the call:
        // a capturing stream would record copies that replay from freed memory
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cs) != cudaSuccess) {
            cudaGetLastError();
            return naFail(SBG_ERR_CUDA, "cudaStreamIsCapturing failed");
        }
        if (cs != cudaStreamCaptureStatusNone)
            return naFail(SBG_ERR_UNSUPPORTED, "the no-alloc realize cannot run on a capturing stream");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return naFail(SBG_ERR_CUDA, "no current CUDA device");
    if ((e = setUpDevice(dev)) != cudaSuccess)
        return naFail(SBG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nb = topo->nb;
    const int nf = (int)topo->fkw.size();
    const int32_t inst[2] = {0, nb};
#define SBG_UP(sym, src, bytes)                                                                   \
    if ((bytes) > 0 && (e = cudaMemcpyToSymbolAsync(sym, src, bytes, 0, cudaMemcpyHostToDevice, s)) != cudaSuccess) \
        return naFail(SBG_ERR_CUDA, std::string("table upload: ") + cudaGetErrorString(e));
    SBG_UP(g_naParent, topo->parent.data(), nb * sizeof(int32_t))
    SBG_UP(g_naInfo, topo->info.data(), nb * sizeof(int32_t))
    SBG_UP(g_naQoff, topo->qoff.data(), nb * sizeof(int32_t))
    SBG_UP(g_naUoff, topo->uoff.data(), nb * sizeof(int32_t))
    const int nmw = topo->maxNonFreeDof <= 1 ? 1 : 3;
    int64_t recSize = 0;
    const std::vector<int32_t> srecPad = paddedRecords(*topo, nmw, &recSize);
    SBG_UP(g_naSrec, srecPad.data(), nb * sizeof(int32_t))
    SBG_UP(g_naFbeg, topo->fbeg.data(), nb * sizeof(int32_t))
    SBG_UP(g_naFcnt, topo->fcnt.data(), nb * sizeof(int32_t))
    SBG_UP(g_naPar, topo->par.data(), topo->par.size() * sizeof(double))
    SBG_UP(g_naFkw, topo->fkw.data(), nf * sizeof(int32_t))
    SBG_UP(g_naFcoef, topo->fcoef.data(), nf * sizeof(double))
    SBG_UP(g_naFq0, topo->fq0.data(), nf * sizeof(double))
    SBG_UP(g_naInst, inst, sizeof inst)
    SBG_UP(g_naGrav, topo->gravity, 3 * sizeof(double))
#undef SBG_UP
    const int64_t slotsFit = (int64_t)kNoAllocScratchBytes / recBytes;
    const int threads = 128;
    // every launched thread owns one scratch slot: nthreads <= slotsFit
    int64_t nthreads = std::min<int64_t>(slotsFit, ninst);
    if (nthreads >= threads) nthreads = (nthreads / threads) * threads;
    const int block = (int)std::min<int64_t>(threads, nthreads);
    const int grid = (int)(nthreads / block);
    const DevTables& T = g_naTables[dev];
    if (nmw == 1)
        realizeNoAllocKernel<1><<<grid, block, 0, s>>>(T, y, ydot, status, g_naScratchPtr[dev], ninst, topo->nq,
                                                       topo->nq + topo->nu, recSize);
    else
        realizeNoAllocKernel<3><<<grid, block, 0, s>>>(T, y, ydot, status, g_naScratchPtr[dev], ninst, topo->nq,
                                                       topo->nq + topo->nu, recSize);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return naFail(SBG_ERR_CUDA, std::string("no-alloc kernel launch: ") + cudaGetErrorString(e));
    return SBG_OK;
}

}  // extern "C"
