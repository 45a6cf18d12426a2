// kpm_step_f64.cu — step-kernel instantiations for double vectors.
#include "kpm_step.cuh"

namespace tbk {

int launch_step_f64(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<double, true>(R, a, first, braket, grid, st) : launch_step<double, false>(R, a, first, braket, grid, st);
}

int occupancy_f64(bool cplx, int R) {
  switch (R) {
    case 1: return cplx ? occupancy_blocks<double, true, 1>() : occupancy_blocks<double, false, 1>();
    case 2: return cplx ? occupancy_blocks<double, true, 2>() : occupancy_blocks<double, false, 2>();
    case 4: return cplx ? occupancy_blocks<double, true, 4>() : occupancy_blocks<double, false, 4>();
    case 8: return cplx ? occupancy_blocks<double, true, 8>() : occupancy_blocks<double, false, 8>();
    case 16: return cplx ? occupancy_blocks<double, true, 16>() : occupancy_blocks<double, false, 16>();
    default: return cplx ? occupancy_blocks<double, true, 32>() : occupancy_blocks<double, false, 32>();
  }
}

}  // namespace tbk
