// hpsi_4x3.cu -- fixed-shape H*psi for the 4x3 lattice (one translation
// unit per shape so the unrolled kernels compile in parallel).
#include "lgt_hpsi_fixed.cuh"

namespace lgt {

cudaError_t launch_hpsi_4x3(const HpsiArgs<float>& a, uint32_t model, cudaStream_t s) {
  return fixed::launch_shape<4, 3, float>(a, model, s);
}

cudaError_t launch_hpsi_4x3(const HpsiArgs<double>& a, uint32_t model, cudaStream_t s) {
  return fixed::launch_shape<4, 3, double>(a, model, s);
}

}  // namespace lgt
