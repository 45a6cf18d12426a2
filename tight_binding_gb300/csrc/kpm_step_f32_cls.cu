// kpm_step_f32_cls.cu — class-form step-kernel instantiations for float vectors
// (rows of a translation-invariant matrix; see kpm_step.cuh, CLS).
#include "kpm_step.cuh"

namespace tbk {

int launch_step_cls_f32(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<float, true, true>(R, a, first, braket, grid, st)
              : launch_step<float, false, true>(R, a, first, braket, grid, st);
}

int occupancy_cls_f32(bool cplx, int R, size_t smem) { return occupancy_r<float, true>(cplx, R, smem); }

}  // namespace tbk
