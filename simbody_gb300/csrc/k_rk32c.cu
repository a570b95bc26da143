// k_rk32c.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with FP64 state accumulation, chain driver.
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB> static void go(const KArgs& a, cudaStream_t s) {
    const int nb = (a.P->nChain + 127) / 128;
    float* fb = static_cast<float*>(a.fbuf);
    float* sc = static_cast<float*>(a.scratch);
    if (a.P->nm == 1)
        rkMersonKernel<float, 1, REF, false, MINB><<<nb, 128, 0, s>>>(*a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc,
                                                                      a.status, a.h, a.nsteps, a.accuracy, a.consTol, a.projectEveryStep);
    else
        rkMersonKernel<float, 3, REF, false, MINB><<<nb, 128, 0, s>>>(*a.T, 0, a.P->nChain, a.ystate, a.time, fb, a.fplane, sc,
                                                                      a.status, a.h, a.nsteps, a.accuracy, a.consTol, a.projectEveryStep);
}

void rk32Chain(const KArgs& a, bool refine, cudaStream_t s) {
    if (refine) { if (a.P->variant == 4) go<true, 4>(a, s); else go<true, 1>(a, s); }
    else { if (a.P->variant == 4) go<false, 4>(a, s); else go<false, 1>(a, s); }
}

}  // namespace sbg
