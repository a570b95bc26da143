// k_r32s.cu -- realize(Acceleration), FP32 recursions (refined or not), for a
// batch whose instances all share one unbranched chain topology without Free
// bodies (the 32-Ball chain benchmark is one): the chain driver with each
// body's scratch-record fields staged through shared memory.
//
// The chain driver walks the bodies of its instance in order (passes 1, 3, 5)
// and in reverse order (passes 2, 4); every pass after the first reads fields
// of the body's record that an earlier pass wrote. Those reads are the
// kernel's long stalls: a warp waits on DRAM at every body. Here the 32
// instances of a warp form one scratch tile (field f of a record is 32
// consecutive floats, one per instance), so the fields a pass reads for one
// body are a few contiguous 128-byte rows of the tile. While the warp
// computes body k, its lanes copy the rows of the next body into the other
// half of a double buffer with cp.async (16 bytes per lane and copy), and
// cp.async.wait_group plus __syncwarp hand it over. The arithmetic and the
// record layout are those of the chain driver, so the results are the same
// bit for bit; only where the loads come from changes. Writes go to the
// records in global memory as before.
//
// Pass read sets (record of N = batch width columns; f = mobility forces,
// eps written by pass 2 and rewritten by pass 4):
//   pass 2  [18,42) pc Gi l a bF             + [69, eDI) H f
//   pass 3  [69, eU0) H f DI G eps           (pc Gi l a bF read directly)
//   pass 4  [27,30) l + [42,54) F_df + [69, eDI) H f + [eG, eEps) G
//   pass 5  [27,30) l + [69, ef) H + [eDI, end) DI G eps udot0
// Pass 1 reads no record.
#include "abi_device.cuh"

namespace sbg {
namespace {

// A pass's read set: up to four field ranges, packed in this order in the
// shared buffer (slot s holds the 32 lanes' values of one field).
template <int A0, int A1, int B0, int B1, int C0, int C1, int D0, int D1> struct StageSet {
    static constexpr int nA = A1 - A0, nB = B1 - B0, nC = C1 - C0, nD = D1 - D0;
    static constexpr int size = nA + nB + nC + nD;
    static __device__ __forceinline__ constexpr int slot(int f) {
        return (f >= A0 && f < A1) ? f - A0
               : (f >= B0 && f < B1) ? nA + f - B0
               : (f >= C0 && f < C1) ? nA + nB + f - C0
               : (f >= D0 && f < D1) ? nA + nB + nC + f - D0
                                     : -1;
    }
};

template <int N> struct Sets {
    static constexpr int ef = kRecH + 6 * N, eDI = ef + N, eG = eDI + N * N, eEps = eG + 6 * N, eU0 = eEps + N,
                         end = eU0 + N;
    using P2 = StageSet<kRecPc, kRecBF + 6, kRecH, eDI, 0, 0, 0, 0>;
    using P3 = StageSet<kRecH, eU0, 0, 0, 0, 0, 0, 0>;
    using P4 = StageSet<kRecL, kRecL + 3, kRecFdf, kRecFdf + 12, kRecH, eDI, eG, eEps>;
    using P5 = StageSet<kRecL, kRecL + 3, kRecH, ef, eDI, end, 0, 0>;
    static constexpr int maxSize = P2::size > P3::size ? (P2::size > P4::size ? (P2::size > P5::size ? P2::size : P5::size)
                                                                               : (P4::size > P5::size ? P4::size : P5::size))
                                                       : (P3::size > P4::size ? (P3::size > P5::size ? P3::size : P5::size)
                                                                               : (P4::size > P5::size ? P4::size : P5::size));
};

// Element f of the current record: from the shared buffer when the pass
// staged it, else from the lane's column of the tile in global memory.
template <class SET> struct ScrStaged {
    float* g;   // lane's column of the tile: element (rec + f) * 32
    float* sm;  // lane's column of the current buffer: slot s at s * 32
    __device__ __forceinline__ float& operator()(int rec, int f) const {
        const int s = SET::slot(f);
        return s >= 0 ? sm[s * kTile] : g[(rec + f) * kTile];
    }
};

__device__ __forceinline__ void cpAsync16(uint32_t dst, const float* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void prefetchL2(const void* p) { asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p)); }
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int K> __device__ __forceinline__ void cpAsyncWait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(K) : "memory"); }

// Copy fields [F0, F1) of the record at recTile (the tile's element of
// field 0 of the record) to slots [S0, ...) of the buffer at byte address sbuf.
template <int F0, int F1, int S0>
__device__ __forceinline__ void stageRange(const float* recTile, uint32_t sbuf, int lane) {
    constexpr int chunks = (F1 - F0) * (kTile / 4);  // 16-byte chunks
#pragma unroll 4
    for (int c = lane; c < chunks; c += 32)
        cpAsync16(sbuf + (uint32_t)((S0 * kTile + 4 * c) * 4), recTile + F0 * kTile + 4 * c);
}
template <class SET, int A0, int A1, int B0, int B1, int C0, int C1, int D0, int D1>
__device__ __forceinline__ void stageAll(StageSet<A0, A1, B0, B1, C0, C1, D0, D1>*, const float* recTile, uint32_t sbuf,
                                         int lane) {
    if constexpr (A1 > A0) stageRange<A0, A1, 0>(recTile, sbuf, lane);
    if constexpr (B1 > B0) stageRange<B0, B1, SET::nA>(recTile, sbuf, lane);
    if constexpr (C1 > C0) stageRange<C0, C1, SET::nA + SET::nB>(recTile, sbuf, lane);
    if constexpr (D1 > D0) stageRange<D0, D1, SET::nA + SET::nB + SET::nC>(recTile, sbuf, lane);
}
template <class SET> __device__ __forceinline__ void stage(const float* recTile, uint32_t sbuf, int lane) {
    stageAll<SET>(static_cast<SET*>(nullptr), recTile, sbuf, lane);
}

// One pass over the bodies in the given direction with the read set SET
// double-buffered: body(lb, S) computes body lb with S addressing its
// staged record (only on lanes that hold an instance).
template <class SET, bool FORWARD, class Body, class Ahead>
__device__ __forceinline__ void stagedPass(const DevTables& T, int body0, int nb, float* tile, float* buf, int lane,
                                           bool valid, Body&& body, Ahead&& ahead) {
    const uint32_t sb0 = (uint32_t)__cvta_generic_to_shared(buf);
    const uint32_t bytes = (uint32_t)(SET::size * kTile * 4);
    auto recOf = [&](int lb) { return tile + (int64_t)T.srec[body0 + lb] * kTile; };
    const int first = FORWARD ? 0 : nb - 1, step = FORWARD ? 1 : -1;
    stage<SET>(recOf(first), sb0, lane);
    cpAsyncCommit();
    for (int k = 0; k < nb; ++k) {
        const int lb = first + step * k;
        if (k + 1 < nb) {
            stage<SET>(recOf(lb + step), sb0 + ((k + 1) & 1) * bytes, lane);
            ahead(lb + step);
        }
        cpAsyncCommit();
        cpAsyncWait<1>();  // this lane's copies of body lb have landed
        __syncwarp();      // ... and every other lane's
        if (valid) {
            const ScrStaged<SET> S{tile + lane, buf + (k & 1) * SET::size * kTile + lane};
            body(lb, S);
        }
        __syncwarp();  // buffer k & 1 is refilled at iteration k + 1
    }
    cpAsyncWait<0>();
    __threadfence_block();  // this pass's record writes, before the next pass's copies of them
    __syncwarp();
}

template <int NM, bool REF, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB)
    realizeStagedKernel(DevTables T, int first, int count, const double* __restrict__ y, double* __restrict__ ydot,
                        float* __restrict__ scratch, int32_t* __restrict__ status) {
    using SS = Sets<NM>;
    extern __shared__ float4 smemRaw[];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int warpFirst = t - lane;
    if (warpFirst >= count) return;  // whole warp beyond the segment
    const bool valid = t < count;
    // lane 0 of a warp holds the first instance of a tile (first is a
    // multiple of 32), whose scratch column is the tile's first
    const int inst0 = T.order[first + warpFirst];
    const int inst = valid ? T.order[first + t] : inst0;
    float* tile = scratch + T.sbase[inst0];
    float* buf = reinterpret_cast<float*>(smemRaw) + (threadIdx.x >> 5) * 2 * SS::maxSize * kTile;
    const int body0 = T.ibody[inst0], nb = T.inb[inst0];
    const YSrc src{y, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    YdOut out{ydot, T.ybase[inst], T.ystride[inst], T.inq[inst]};
    const V3<float> g = mk3(float(T.grav[3 * inst]), float(T.grav[3 * inst + 1]), float(T.grav[3 * inst + 2]));
    const float* PT = T.par32;
    const ScrTiled<float> SG{tile + lane};
    // state rows of the tile (element k of its 32 instances: 256 bytes at
    // ybase0 + 32 k), prefetched into L2 one body ahead
    const double* ytile = y + T.ybase[inst0];
    const int nq0 = T.inq[inst0];
    auto aheadY = [&](int lb) {
        const int row = body0 + lb;
        const int n = (T.info[row] >> 4) & 15, nqb = (T.info[row] & 15) == T_BALL ? 4 : n;
        const int line = lane >> 1, half = lane & 1;  // two 128-byte lines per element
        if (line < nqb) prefetchL2(ytile + (T.qoff[row] + line) * kTile + 16 * half);
        else if (line < nqb + n) prefetchL2(ytile + (nq0 + T.uoff[row] + line - nqb) * kTile + 16 * half);
    };
    {  // pass 1: kinematics carried along the chain, nothing read back
        Kin<float> carry = groundKin<float>();
        for (int lb = 0; lb < nb; ++lb) {
            if (lb + 1 < nb) aheadY(lb + 1);
            if (valid) carry = body1<float, NM>(T, body0 + lb, T.srec[body0 + lb], SG, src, out, g, carry);
        }
    }
    __threadfence_block();
    __syncwarp();
    bool ok = true;
    {  // pass 2
        C2<float> carry = zeroC2<float>();
        stagedPass<typename SS::P2, false>(T, body0, nb, tile, buf, lane, valid, [&](int lb, const auto& S) {
            const int row = body0 + lb;
            const int n = (T.info[row] >> 4) & 15;
            C2<float> in = zeroC2<float>();
            if (lb != nb - 1) addC2(in, carry);  // as the chain driver: zero + carry
            C2<float> outC;
            ok &= body2<float, NM>(T, row, T.srec[row], n, S, PT[(int64_t)row * kParamStride], in, outC);
            carry = outC;
        }, [](int) {});
    }
    {  // pass 3
        A3<float> carry{};
        stagedPass<typename SS::P3, true>(T, body0, nb, tile, buf, lane, valid, [&](int lb, const auto& S) {
            const int row = body0 + lb;
            const int n = (T.info[row] >> 4) & 15;
            carry = body3<float, NM, REF>(T, row, T.srec[row], n, S, out, lb == 0 ? A3<float>{} : carry, lb > 0);
        }, [&](int lb) {  // the fields read directly (pc Gi l a bF): one 128-byte row each
            if (lane < kRecBF + 6 - kRecPc) prefetchL2(tile + ((int64_t)T.srec[body0 + lb] + kRecPc + lane) * kTile);
        });
    }
    if constexpr (REF) {
        {  // pass 4
            C4 carry = zeroC4();
            stagedPass<typename SS::P4, false>(T, body0, nb, tile, buf, lane, valid, [&](int lb, const auto& S) {
                const int row = body0 + lb;
                const int n = (T.info[row] >> 4) & 15;
                const int rec = T.srec[row];
                const C4 own{ldDF3(S, rec, kRecFdf), ldDF3(S, rec, kRecFdf + 6), z3<float>(), z3<float>()};
                carry = body4<NM>(T, row, rec, n, S, own, lb == nb - 1 ? zeroC4() : carry);
            }, [](int) {});
        }
        {  // pass 5
            A3<float> carry{};
            stagedPass<typename SS::P5, true>(T, body0, nb, tile, buf, lane, valid, [&](int lb, const auto& S) {
                const int row = body0 + lb;
                const int n = (T.info[row] >> 4) & 15;
                carry = body5<NM>(T, row, T.srec[row], n, S, out, lb == 0 ? A3<float>{} : carry, lb > 0);
            }, [](int) {});
        }
    }
    if (!valid) return;
    int st = ok ? 0 : SBG_INST_SINGULAR_D;
    if constexpr (REF) st |= illConditioned<false>(T, out, Slot{inst, 0, 1, 0u});
    if (!out.finite) st |= SBG_INST_NONFINITE;
    status[inst] = st;
}

template <int NM, bool REF> void goStaged(const KArgs& a, cudaStream_t s) {
    constexpr int BS = 64, MINB = 7;
    const size_t smem = (size_t)(BS / 32) * 2 * Sets<NM>::maxSize * kTile * sizeof(float);
    static bool attr = false;  // one-time opt-in above the default 48 KB (not needed at these sizes)
    if (!attr && smem > 48 * 1024) {
        cudaFuncSetAttribute(realizeStagedKernel<NM, REF, BS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = true;
    }
    const int grid = (a.P->nChain + BS - 1) / BS;
    if (grid == 0) return;
    realizeStagedKernel<NM, REF, BS, MINB><<<grid, BS, smem, s>>>(*a.T, a.P->chainFirst, a.P->nChain, a.y, a.ydot,
                                                                  static_cast<float*>(a.scratch), a.status);
}

}  // namespace

void realize32ChainStaged(const KArgs& a, bool refine, cudaStream_t s) {
    if (a.P->nm == 1) {
        if (refine) goStaged<1, true>(a, s); else goStaged<1, false>(a, s);
    } else {
        if (refine) goStaged<3, true>(a, s); else goStaged<3, false>(a, s);
    }
    if (refine) realizeFallback(a, false, s);
}

}  // namespace sbg
