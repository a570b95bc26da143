// rk32c_launch.cuh -- the launcher of the FP32 chain-driver RK-Merson kernels,
// shared by the translation units that instantiate its refined (k_rk32cr.cu)
// and unrefined (k_rk32c.cu) forms, which compile in parallel. Occupancy
// variants as in k_r32c.cu (1, 4: 128-thread blocks; 7: 64-thread blocks).
#pragma once
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB, int BS> static void rk32ChainGo(const KArgs& a, cudaStream_t s) {
    const Launch1D L = spread(a.P->nChain, BS);
    float* fb = static_cast<float*>(a.fbuf);
    float* sc = static_cast<float*>(a.scratch);
    if (a.P->nm == 1)
        rkMersonKernel<float, 1, REF, false, MINB, false, BS><<<L.grid, L.block, 0, s>>>(
            *a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc, a.status, a.h, a.step, a.accuracy, a.consTol,
            a.projectEveryStep);
    else
        rkMersonKernel<float, 3, REF, false, MINB, false, BS><<<L.grid, L.block, 0, s>>>(
            *a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc, a.status, a.h, a.step, a.accuracy, a.consTol,
            a.projectEveryStep);
}

template <bool REF> static void rk32ChainPick(const KArgs& a, cudaStream_t s) {
    if (a.P->variant == 4) rk32ChainGo<REF, 4, 128>(a, s);
    else if (a.P->variant >= 7) rk32ChainGo<REF, 7, 64>(a, s);  // 8: realize only
    else rk32ChainGo<REF, 1, 128>(a, s);
}

// k_rk32cr.cu: the refined (mixed) form.
void rk32ChainRefined(const KArgs& a, cudaStream_t s);

}  // namespace sbg
