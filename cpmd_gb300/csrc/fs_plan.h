// Four-step FFT plans shared by the host (twiddle tables) and the kernels:
// N = N1 * N2 and the number of lines L one CTA transforms.
#pragma once

namespace gbcp {

__host__ __device__ constexpr int fs_n1(int n) {
  return n == 32 ? 4 : n == 36 ? 6 : n == 40 ? 8 : n == 48 ? 4 : n == 60 ? 4 : n == 64 ? 8 : n == 72 ? 6
       : n == 80 ? 8 : n == 96 ? 8 : n == 120 ? 8 : n == 144 ? 12 : n == 240 ? 12 : 0;
}
__host__ __device__ constexpr int fs_lines(int n) {
  return n == 32 ? 64 : n == 36 ? 42 : n == 40 ? 32 : n == 48 ? 64 : n == 60 ? 64 : n == 64 ? 32 : n == 72 ? 42
       : n == 80 ? 32 : n == 96 ? 32 : n == 120 ? 32 : n == 144 ? 21 : n == 240 ? 21 : 0;
}

}  // namespace gbcp
