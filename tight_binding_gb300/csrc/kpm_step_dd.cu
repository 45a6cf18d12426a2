// kpm_step_dd.cu — step-kernel instantiations for dd vectors.
#include "kpm_step.cuh"

namespace tbk {

int launch_step_dd(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<dd, true>(R, a, first, braket, grid, st) : launch_step<dd, false>(R, a, first, braket, grid, st);
}

int occupancy_dd(bool cplx, int R) { return occupancy_r<dd, false>(cplx, R, 0); }

}  // namespace tbk
