// k_fallback.cu -- FP64 recomputation of the mixed realize's ill-conditioned
// instances (realizeFallbackKernel), one launch per segment after its mixed
// kernel on the same stream.
#include "abi_device.cuh"

namespace sbg {

void realizeFallback(const KArgs& a, bool group, cudaStream_t s) {
    if (!a.T->scratch64) return;
    if (group) {
        const int first = a.P->nChain + a.P->nLoop, count = a.T->ninst - first;
        if (count <= 0) return;
        realizeFallbackKernel<3, true><<<(count + 127) / 128, 128, 0, s>>>(*a.T, first, count, a.y, a.ydot, a.status);
    } else {
        const int count = a.P->nChain;
        if (count <= 0) return;
        if (a.P->nm == 1)
            realizeFallbackKernel<1, false><<<(count + 127) / 128, 128, 0, s>>>(*a.T, a.P->chainFirst, count, a.y,
                                                                               a.ydot, a.status);
        else
            realizeFallbackKernel<3, false><<<(count + 127) / 128, 128, 0, s>>>(*a.T, a.P->chainFirst, count, a.y,
                                                                               a.ydot, a.status);
    }
}

}  // namespace sbg
