// kpm_step_f64_cls.cu — class-form step-kernel instantiations for double vectors
// (rows of a translation-invariant matrix; see kpm_step.cuh, CLS).
#include "kpm_step.cuh"

namespace tbk {

int launch_step_cls_f64(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<double, true, true>(R, a, first, braket, grid, st)
              : launch_step<double, false, true>(R, a, first, braket, grid, st);
}

int occupancy_cls_f64(bool cplx, int R, size_t smem) { return occupancy_r<double, true>(cplx, R, smem); }

}  // namespace tbk
