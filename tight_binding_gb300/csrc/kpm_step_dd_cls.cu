// kpm_step_dd_cls.cu — class-form step-kernel instantiations for dd vectors
// (rows of a translation-invariant matrix; see kpm_step.cuh, CLS).
#include "kpm_step.cuh"

namespace tbk {

int launch_step_cls_dd(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<dd, true, true>(R, a, first, braket, grid, st)
              : launch_step<dd, false, true>(R, a, first, braket, grid, st);
}

int occupancy_cls_dd(bool cplx, int R, size_t smem) { return occupancy_r<dd, true>(cplx, R, smem); }

}  // namespace tbk
