// kpm_step_f32.cu — step-kernel instantiations for float vectors.
#include "kpm_step.cuh"

namespace tbk {

int launch_step_f32(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<float, true>(R, a, first, braket, grid, st) : launch_step<float, false>(R, a, first, braket, grid, st);
}

int occupancy_f32(bool cplx, int R) { return occupancy_r<float, false>(cplx, R, 0); }

}  // namespace tbk
