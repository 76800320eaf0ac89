// Row pairing of the FP32 interpolation kernel (imaging.cu, fi_out_kernel): with the
// centred row coordinate y' = Y + (Fy-Ly)/2 - Fy/2, one set of sums over the band rows
// serves the base row b = |y'| and gives rows y' = +b and y' = -b.  Plain C++ (host and
// device), so the pairing is also checked on the CPU.
#pragma once

#ifdef __CUDACC__
#define LITHO_FO_HD __host__ __device__
#else
#define LITHO_FO_HD
#endif

namespace litho {

// offset from the image row Y to y'
LITHO_FO_HD inline int fo_oy(int Ly, int Fy) { return (Fy - Ly) / 2 - Fy / 2; }

// base rows of a geometry: b = 0 .. max |y'| over the image rows
LITHO_FO_HD inline int fo_nbase(int Ly, int Fy) {
  const long long oy = fo_oy(Ly, Fy);
  const long long lo = oy < 0 ? -oy : oy, hi = oy + Ly - 1 < 0 ? -(oy + Ly - 1) : oy + Ly - 1;
  return (int)(lo > hi ? lo : hi) + 1;
}

// image row of base row b and sign sgn (0: y' = +b, 1: y' = -b), or -1 where that row is not
// in the image (or is y' = 0 a second time)
LITHO_FO_HD inline int fo_row(int b, int sgn, int Ly, int Fy) {
  if (sgn == 1 && b == 0) return -1;
  const int Y = (sgn == 0 ? b : -b) - fo_oy(Ly, Fy);
  return Y >= 0 && Y < Ly ? Y : -1;
}

}  // namespace litho
