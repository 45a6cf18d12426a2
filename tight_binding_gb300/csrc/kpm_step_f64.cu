// kpm_step_f64.cu — step-kernel instantiations for double vectors.
#include "kpm_step.cuh"

namespace tbk {

int launch_step_f64(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<double, true>(R, a, first, braket, grid, st) : launch_step<double, false>(R, a, first, braket, grid, st);
}

int occupancy_f64(bool cplx, int R) { return occupancy_r<double, false>(cplx, R, 0); }

}  // namespace tbk
