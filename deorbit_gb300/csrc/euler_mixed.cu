// euler_mixed.cu -- the mixed form's Lop kernels of the Eulerian grid
// hydrocode: primitives, face fluxes and right-hand-side sources in FP32
// (the arithmetic of the reference's own GPU solver), compiled with fused
// multiply-adds; the FP64 state, stages and control live in euler.cu.
#include "euler_kernels.cuh"

namespace deu {

void enqueue_lop_f32(const P& p, const Fields& s, PrimT<float> W, const double* af, FacesT<float> F, Rhs d,
                     const Ctl* ctl, cudaStream_t st) {
    enqueue_lop_t<float>(p, s, W, af, F, d, ctl, st);
}

}  // namespace deu
