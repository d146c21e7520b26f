// mhd_fp32.cu — chosen form: reconstruction, Riemann solver, characteristic
// and EMF arithmetic in FP32; accumulation into the FP64 state.  Built with
// the default contraction (FMA) enabled.
#include "mhd_sweep_impl.cuh"

namespace mhd {
cudaError_t sweep_fp32(int dir, const SweepArgs &a, cudaStream_t s) { return launch_sweep<float>(dir, a, s); }
cudaError_t emf_fp32(int e, const CTArgs &a, cudaStream_t s) { return launch_emf<float>(e, a, s); }
}  // namespace mhd
