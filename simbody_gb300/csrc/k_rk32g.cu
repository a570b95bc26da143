// k_rk32g.cu -- fixed-step RK-Merson persistent kernel instantiations, FP32
// recursions with FP64 state accumulation, level-parallel driver.
#include "abi_device.cuh"

namespace sbg {

template <bool REF, int MINB> static void go(const KArgs& a, cudaStream_t s) {
    rkMersonKernel<float, 3, REF, true, MINB><<<a.P->nGroupBlocks, 128, 0, s>>>(
        *a.T, a.P->groupFirst, 0, a.ystate, a.time, static_cast<float*>(a.fbuf), a.fplane, static_cast<float*>(a.scratch), a.status,
        a.h, a.step, a.accuracy, a.consTol, a.projectEveryStep);
}

void rk32Group(const KArgs& a, bool refine, cudaStream_t s) {
    if (refine) { if (a.P->variant >= 4) go<true, 4>(a, s); else go<true, 1>(a, s); }
    else { if (a.P->variant >= 4) go<false, 4>(a, s); else go<false, 1>(a, s); }
}

}  // namespace sbg
