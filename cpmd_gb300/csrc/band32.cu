// FP32 instantiation of the band loop (mixed mode: FP32 FFT and V*psi,
// FP64 density accumulation, decode and c2 accumulation).
#include "band_impl.cuh"

namespace gbcp {
int band_rhoofr_fp32(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho,
                     double* kpart) {
  return band::rhoofr_t<float>(c, c0, ldc, nstate, f, rho, kpart);
}
int band_zinv_blocks_fp32(const Ctx& c) { return band::kin_blocks<float>(c); }
int band_vpsi_fp32(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f,
                   const double* vpot, int nstate) {
  return band::vpsi_t<float>(c, c0, ldc, c2, ldc2, f, vpot, nstate);
}
}  // namespace gbcp
