// r32c_launch.cuh -- the launcher of the FP32 chain-driver realize kernels,
// shared by the translation units that instantiate its refined (k_r32cr.cu)
// and unrefined (k_r32c.cu) forms, which compile in parallel. Occupancy
// variants: 1 = 128-thread blocks with every register the code wants; 4 =
// 128-thread blocks, at most 128 registers (4 blocks per SM); 7 = 64-thread
// blocks, at most 144 registers (7 blocks per SM), which keeps a batch of
// 65,536 one-thread instances in a single balanced wave over 152 SMs; 8 =
// 7 with the records staged through shared memory (k_r32s.cu), for a batch
// of one shared chain topology without Free bodies.
#pragma once
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB, int BS> static void r32ChainGo(const KArgs& a, cudaStream_t s) {
    const Launch1D L = spread(a.P->nChain, BS);
    float* sc = static_cast<float*>(a.scratch);
    if (a.P->nm == 1)
        realizeKernel<float, 1, REF, false, MINB, false, BS><<<L.grid, L.block, 0, s>>>(*a.T, a.P->chainFirst, a.P->nChain, a.y, a.ydot, sc, a.status);
    else
        realizeKernel<float, 3, REF, false, MINB, false, BS><<<L.grid, L.block, 0, s>>>(*a.T, a.P->chainFirst, a.P->nChain, a.y, a.ydot, sc, a.status);
}

template <bool REF> static void r32ChainPick(const KArgs& a, cudaStream_t s) {
    if (a.P->variant == 4) r32ChainGo<REF, 4, 128>(a, s);
    else if (a.P->variant >= 7) r32ChainGo<REF, 7, 64>(a, s);
    else r32ChainGo<REF, 1, 128>(a, s);
}

// k_r32cr.cu: the refined (mixed) form.
void realize32ChainRefined(const KArgs& a, cudaStream_t s);

}  // namespace sbg
