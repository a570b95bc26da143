// k_rk32c.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with FP64 state accumulation, chain driver. Occupancy variants
// as in k_r32c.cu (1, 4: 128-thread blocks; 7: 64-thread blocks, 144
// registers).
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB, int BS> static void go(const KArgs& a, cudaStream_t s) {
    const int nb = (a.P->nChain + BS - 1) / BS;
    float* fb = static_cast<float*>(a.fbuf);
    float* sc = static_cast<float*>(a.scratch);
    if (a.P->nm == 1)
        rkMersonKernel<float, 1, REF, false, MINB, false, BS><<<nb, BS, 0, s>>>(
            *a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc, a.status, a.h, a.nsteps, a.accuracy, a.consTol,
            a.projectEveryStep);
    else
        rkMersonKernel<float, 3, REF, false, MINB, false, BS><<<nb, BS, 0, s>>>(
            *a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc, a.status, a.h, a.nsteps, a.accuracy, a.consTol,
            a.projectEveryStep);
}

template <bool REF> static void pick(const KArgs& a, cudaStream_t s) {
    if (a.P->variant == 4) go<REF, 4, 128>(a, s);
    else if (a.P->variant == 7) go<REF, 7, 64>(a, s);
    else go<REF, 1, 128>(a, s);
}

void rk32Chain(const KArgs& a, bool refine, cudaStream_t s) {
    if (refine) pick<true>(a, s);
    else pick<false>(a, s);
}

}  // namespace sbg
