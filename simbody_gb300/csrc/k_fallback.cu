// k_fallback.cu -- FP64 work of the mixed form's ill-conditioned instances:
// the realize's recomputation (realizeFallbackKernel, one launch per segment
// after its mixed kernel on the same stream) and the FP64 steps of a mixed
// batch integration (rkFp64List).
#include "abi_device.cuh"

namespace sbg {

void realizeFallback(const KArgs& a, bool group, cudaStream_t s) {
    if (!a.T->scratch64) return;
    if (group) {
        const int first = a.P->nChain + a.P->nLoop, count = a.T->ninst - first;
        if (count <= 0) return;
        const Launch1D L = spread(count, 128);
        realizeFallbackKernel<3, true><<<L.grid, L.block, 0, s>>>(*a.T, first, count, a.y, a.ydot, a.status);
    } else {
        const int count = a.P->nChain;
        if (count <= 0) return;
        const Launch1D L = spread(count, 128);
        if (a.P->nm == 1)
            realizeFallbackKernel<1, false><<<L.grid, L.block, 0, s>>>(*a.T, a.P->chainFirst, count, a.y,
                                                                               a.ydot, a.status);
        else
            realizeFallbackKernel<3, false><<<L.grid, L.block, 0, s>>>(*a.T, a.P->chainFirst, count, a.y,
                                                                               a.ydot, a.status);
    }
}

// The FP64 steps of the instances in FP64 mode at a one-step launch of a
// mixed batch integration: rkMersonKernel with LIST on FP64 records at
// rowsBase per instance into rows. lanes 1: one thread per instance, the
// one-thread driver on contiguous records (the batch's record offsets);
// otherwise kFbLanes lanes per instance, the level-parallel driver on the
// field-major layout. The grid covers every instance; threads past the list's
// length return at once.
void rkFp64List(const KArgs& a, const int64_t* rowsBase, double* rows, int lanes, cudaStream_t s) {
    DevTables T = *a.T;
    if (!T.fbList || T.ninst <= 0) return;
    T.sbase = rowsBase;
    if (lanes == 1) {
        const int nb = (T.ninst + 127) / 128;
        if (a.P->nm == 1)
            rkMersonKernel<double, 1, false, false, 1, false, 128, true><<<nb, 128, 0, s>>>(
                T, 0, 0, a.ystate, a.time, T.fbuf64, a.fplane, rows, a.status, a.h, a.step, a.accuracy, a.consTol,
                a.projectEveryStep);
        else
            rkMersonKernel<double, 3, false, false, 1, false, 128, true><<<nb, 128, 0, s>>>(
                T, 0, 0, a.ystate, a.time, T.fbuf64, a.fplane, rows, a.status, a.h, a.step, a.accuracy, a.consTol,
                a.projectEveryStep);
        return;
    }
    const int nb = (int)(((int64_t)T.ninst * kFbLanes + 127) / 128);
    rkMersonKernel<double, 3, false, true, 1, false, 128, true><<<nb, 128, 0, s>>>(
        T, 0, 0, a.ystate, a.time, T.fbuf64, a.fplane, rows, a.status, a.h, a.step, a.accuracy, a.consTol,
        a.projectEveryStep);
}

}  // namespace sbg
