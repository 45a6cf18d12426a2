// kpm_step_dd.cu — step-kernel instantiations for dd vectors.
#include "kpm_step.cuh"

namespace tbk {

int launch_step_dd(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<dd, true>(R, a, first, braket, grid, st) : launch_step<dd, false>(R, a, first, braket, grid, st);
}

int occupancy_dd(bool cplx, int R) {
  switch (R) {
    case 1: return cplx ? occupancy_blocks<dd, true, 1>() : occupancy_blocks<dd, false, 1>();
    case 2: return cplx ? occupancy_blocks<dd, true, 2>() : occupancy_blocks<dd, false, 2>();
    case 4: return cplx ? occupancy_blocks<dd, true, 4>() : occupancy_blocks<dd, false, 4>();
    case 8: return cplx ? occupancy_blocks<dd, true, 8>() : occupancy_blocks<dd, false, 8>();
    case 16: return cplx ? occupancy_blocks<dd, true, 16>() : occupancy_blocks<dd, false, 16>();
    default: return cplx ? occupancy_blocks<dd, true, 32>() : occupancy_blocks<dd, false, 32>();
  }
}

}  // namespace tbk
