// kpm_step_f32.cu — step-kernel instantiations for float vectors.
#include "kpm_step.cuh"

namespace tbk {

int launch_step_f32(bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  return cplx ? launch_step<float, true>(R, a, first, braket, grid, st) : launch_step<float, false>(R, a, first, braket, grid, st);
}

int occupancy_f32(bool cplx, int R) {
  switch (R) {
    case 1: return cplx ? occupancy_blocks<float, true, 1>() : occupancy_blocks<float, false, 1>();
    case 2: return cplx ? occupancy_blocks<float, true, 2>() : occupancy_blocks<float, false, 2>();
    case 4: return cplx ? occupancy_blocks<float, true, 4>() : occupancy_blocks<float, false, 4>();
    case 8: return cplx ? occupancy_blocks<float, true, 8>() : occupancy_blocks<float, false, 8>();
    case 16: return cplx ? occupancy_blocks<float, true, 16>() : occupancy_blocks<float, false, 16>();
    default: return cplx ? occupancy_blocks<float, true, 32>() : occupancy_blocks<float, false, 32>();
  }
}

}  // namespace tbk
