// FP64 instantiation of the band loop (plain FP64 drop-in).
#include "band_impl.cuh"

namespace gbcp {
int band_rhoofr_fp64(Ctx& c, const cx<double>* c0, int ldc, int nstate, const double* f, double* rho,
                     double* kpart) {
  return band::rhoofr_t<double>(c, c0, ldc, nstate, f, rho, kpart);
}
int band_zinv_blocks_fp64(const Ctx& c) { return band::kin_blocks<double>(c); }
int band_vpsi_fp64(Ctx& c, const cx<double>* c0, int ldc, cx<double>* c2, int ldc2, const double* f,
                   const double* vpot, int nstate) {
  return band::vpsi_t<double>(c, c0, ldc, c2, ldc2, f, vpot, nstate);
}
}  // namespace gbcp
