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

// x-stage exchange layout: element (k1, n2) of line l at l*XS + k1*XP + n2.
// The x-stage thread maps are line-major on both sides (coalesced rows of the
// mesh), so an odd line stride alone leaves 2- to 8-way bank conflicts; these
// pitch/stride pairs make both maps conflict-free for 8-byte elements (found
// by an exact count of distinct addresses per bank residue over each warp).
__host__ __device__ constexpr int fs_xpitch(int n) {
  return n == 32 ? 9 : n == 36 ? 9 : n == 40 ? 6 : n == 48 ? 13 : n == 60 ? 20 : n == 64 ? 9 : n == 72 ? 13
       : n == 80 ? 10 : n == 96 ? 13 : n == 120 ? 18 : n == 144 ? 13 : n == 240 ? 23 : 0;
}
__host__ __device__ constexpr int fs_xstride(int n) {
  return n == 32 ? 36 : n == 36 ? 54 : n == 40 ? 53 : n == 48 ? 60 : n == 60 ? 95 : n == 64 ? 72 : n == 72 ? 78
       : n == 80 ? 85 : n == 96 ? 108 : n == 120 ? 159 : n == 144 ? 156 : n == 240 ? 276 : 0;
}

}  // namespace gbcp
