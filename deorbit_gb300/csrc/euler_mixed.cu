// euler_mixed.cu -- the mixed form's kernels of the Eulerian grid hydrocode:
// primitives, face fluxes, right-hand-side sources, the yield surface, damage
// growth and the CFL speed in FP32 (the arithmetic of the reference's own GPU
// solver), compiled with fused multiply-adds; the FP64 state updates and the
// step control are shared with the FP64 form (euler.cu).
#include "euler_kernels.cuh"

namespace deu {

cudaError_t enqueue_lop_f32(const P& p, const Fields& s, PrimT<float> W, const double* af, FacesT<float> F, Rhs d,
                            const Ctl* ctl, cudaStream_t st, const FaceFork* fork) {
    return enqueue_lop_t<float>(p, s, W, af, F, d, ctl, st, fork);
}

void enqueue_maxspeed_f32(const P& p, const Fields& g, Ctl* ctl, cudaStream_t st) {
    enqueue_maxspeed_t<float>(p, g, ctl, st);
}

void enqueue_predict_f32(const P& p, const Fields& g, const Fields& g1, Rhs d, const Ctl* ctl, cudaStream_t st) {
    enqueue_predict_t<float>(p, g, g1, d, ctl, st);
}

void enqueue_correct_f32(const P& p, const Fields& g, const Fields& g1, Rhs d, const Ctl* ctl, cudaStream_t st,
                         int stage) {
    enqueue_correct_t<float>(p, g, g1, d, ctl, st, stage);
}

}  // namespace deu
