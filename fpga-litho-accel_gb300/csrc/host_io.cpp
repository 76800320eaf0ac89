// Host-side helpers of the C ABI: source and mask generators and the BIN /
// kernel_info.txt formats of the reference (validation/golden/src/common/).
// No GPU work here.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "../../include/litho_gb300.h"

namespace {

// radius in pixels: float(param) * int((S-1)/2), truncated (source.cpp:6-7)
int rad_px(float v, int S) { return (int)(v * (float)((S - 1) / 2)); }

}  // namespace

extern "C" {

int litho_create_source(float* src, int S, int type, const float* prm, int normalize) {
  if (src == nullptr || S < 1) return LITHO_ERR_ARG;
  const int n = S * S;
  for (int i = 0; i < n; ++i) src[i] = 0.f;
  const int c = (S - 1) / 2;
  switch (type) {
    case LITHO_SRC_ANNULAR: {  // common/source.cpp:5-23
      if (!prm) return LITHO_ERR_ARG;
      const int ri = rad_px(prm[0], S), ro = rad_px(prm[1], S);
      for (int y = 0; y < S; ++y)
        for (int x = 0; x < S; ++x) {
          const double d = std::sqrt(std::pow(x - c, 2) + std::pow(y - c, 2));
          src[y * S + x] = (d >= ri && d <= ro) ? 1.f : 0.f;
        }
      break;
    }
    case LITHO_SRC_CROSS_QUADRUPOLE: {  // common/source.cpp:25-56 (radius, offset)
      if (!prm) return LITHO_ERR_ARG;
      const int rad = rad_px(prm[0], S), off = rad_px(prm[1], S);
      const int cs[4][2] = {{c, c + off}, {c, c - off}, {c + off, c}, {c - off, c}};
      for (int y = 0; y < S; ++y)
        for (int x = 0; x < S; ++x)
          for (int i = 0; i < 4; ++i) {
            const double dx = x - cs[i][0], dy = y - cs[i][1];
            if (std::sqrt(dx * dx + dy * dy) <= rad) {
              src[y * S + x] = 1.f;
              break;
            }
          }
      break;
    }
    case LITHO_SRC_DIPOLE: {  // common/source.cpp:58-87 (radius, offset, onXAxis); centre S/2
      if (!prm) return LITHO_ERR_ARG;
      const int rad = rad_px(prm[0], S), off = rad_px(prm[1], S);
      const bool onx = prm[2] != 0.f;
      const int cx = S / 2, cy = S / 2;
      const int cs[2][2] = {{cx + (onx ? off : 0), cy + (onx ? 0 : off)}, {cx - (onx ? off : 0), cy - (onx ? 0 : off)}};
      for (int y = 0; y < S; ++y)
        for (int x = 0; x < S; ++x)
          for (int i = 0; i < 2; ++i) {
            const double dx = x - cs[i][0], dy = y - cs[i][1];
            if (std::sqrt(dx * dx + dy * dy) <= rad) {
              src[y * S + x] = 1.f;
              break;
            }
          }
      break;
    }
    case LITHO_SRC_POINT: {  // common/source.cpp:121-128 (x, y)
      if (!prm) return LITHO_ERR_ARG;
      int px = (int)std::round(prm[0] * S / 2.0 + S / 2.0);
      int py = (int)std::round(-1 * prm[1] * S / 2.0 + S / 2.0);
      if (prm[0] >= 0) px -= 1;
      if (-1 * prm[1] >= 0) py -= 1;
      if (px < 0 || py < 0 || px >= S || py >= S) return LITHO_ERR_ARG;
      src[py * S + px] = 1.f;
      break;
    }
    case LITHO_SRC_KEEP:  // caller filled src (imported source): normalise only
      return LITHO_ERR_ARG;
    default:
      return LITHO_ERR_ARG;
  }
  if (normalize) litho_normalize_source(src, S);
  return LITHO_OK;
}

int litho_normalize_source(float* src, int S) {  // common/source.cpp:89-103: sequential float sum
  if (src == nullptr || S < 1) return LITHO_ERR_ARG;
  float sum = 0.f;
  for (int i = 0; i < S * S; ++i) sum += src[i];
  if (sum != 0.f)
    for (int i = 0; i < S * S; ++i) src[i] /= sum;
  return LITHO_OK;
}

int litho_create_linespace(float* msk, int sizeX, int sizeY, int lineWidth, int spaceWidth, int horizontal) {
  // common/mask.cpp:5-29
  if (!msk || sizeX < 1 || sizeY < 1 || lineWidth < 0 || spaceWidth < 0 || lineWidth + spaceWidth < 1)
    return LITHO_ERR_ARG;
  const int period = lineWidth + spaceWidth;
  for (int y = 0; y < sizeY; ++y)
    for (int x = 0; x < sizeX; ++x) msk[y * sizeX + x] = (((horizontal ? y : x) % period) < lineWidth) ? 1.f : 0.f;
  return LITHO_OK;
}

int litho_place_mask(const float* in, int maskX, int maskY, float dose, float* out, int Lx, int Ly) {
  // common/mask.cpp:52-59: centre a maskX x maskY pattern in the Lx x Ly period, times dose
  if (!in || !out || maskX < 1 || maskY < 1 || maskX > Lx || maskY > Ly) return LITHO_ERR_ARG;
  for (int i = 0; i < Lx * Ly; ++i) out[i] = 0.f;
  const int oy = (Ly - maskY) / 2, ox = (Lx - maskX) / 2;
  for (int y = 0; y < maskY; ++y)
    for (int x = 0; x < maskX; ++x) out[(y + oy) * Lx + x + ox] = in[y * maskX + x] * dose;
  return LITHO_OK;
}

int litho_write_bin(const char* path, const float* data, long long n) {
  // common/file_io.cpp:137-150: raw little-endian float32, no header
  if (!path || (!data && n > 0) || n < 0) return LITHO_ERR_ARG;
  std::ofstream f(path, std::ios::binary);
  if (!f) return LITHO_ERR_IO;
  f.write(reinterpret_cast<const char*>(data), (std::streamsize)(n * sizeof(float)));
  return f ? LITHO_OK : LITHO_ERR_IO;
}

int litho_read_bin(const char* path, float* data, long long n) {
  // common/file_io.cpp:232-259: a size mismatch is a warning; the array is
  // truncated or zero-padded to n floats
  if (!path || !data || n < 0) return LITHO_ERR_ARG;
  std::ifstream f(path, std::ios::binary | std::ios::ate);
  if (!f) return LITHO_ERR_IO;
  const long long bytes = (long long)f.tellg();
  f.seekg(0);
  const long long have = bytes / (long long)sizeof(float);
  const long long take = have < n ? have : n;
  f.read(reinterpret_cast<char*>(data), (std::streamsize)(take * sizeof(float)));
  if (!f) return LITHO_ERR_IO;
  for (long long i = take; i < n; ++i) data[i] = 0.f;
  if (bytes != n * (long long)sizeof(float))
    fprintf(stderr, "Warning: File size (%lld bytes) does not match the expected data size (%lld bytes)\n", bytes,
            n * (long long)sizeof(float));
  return LITHO_OK;
}

int litho_write_kernel_info(const char* path, int krnX, int krnY, int nk, const float* scales) {
  // common/file_io.cpp:262-280 (the format litho.cpp writes, not the host tool's)
  if (!path || !scales || nk < 0) return LITHO_ERR_ARG;
  FILE* f = fopen(path, "w");
  if (!f) return LITHO_ERR_IO;
  fprintf(f, "# Kernel Information\n## Kernel Size and Count\n- Kernel Size: %dx%d\n- Number of Kernels: %d\n",
          krnX, krnY, nk);
  fprintf(f, "## Eigenvalues of Each Kernel\n");
  for (int i = 0; i < nk; ++i) fprintf(f, "Eigenvalue %d: %g\n", i, (double)scales[i]);
  return fclose(f) == 0 ? LITHO_OK : LITHO_ERR_IO;
}

int litho_read_kernel_info(const char* path, int* krnX, int* krnY, int* nk, float* scales, int cap) {
  // common/file_io.cpp:282-307
  if (!path || !krnX || !krnY || !nk) return LITHO_ERR_ARG;
  std::ifstream f(path);
  if (!f) return LITHO_ERR_IO;
  std::string line;
  *nk = 0;
  while (std::getline(f, line)) {
    if (line.find("Kernel Size:") != std::string::npos) {
      sscanf(line.c_str(), "- Kernel Size: %dx%d", krnX, krnY);
    } else if (line.find("Number of Kernels:") != std::string::npos) {
      sscanf(line.c_str(), "- Number of Kernels: %d", nk);
    } else if (line.find("Eigenvalue") != std::string::npos) {
      int idx = -1;
      double v = 0.0;
      if (sscanf(line.c_str(), "Eigenvalue %d: %lf", &idx, &v) == 2 && scales && idx >= 0 && idx < cap &&
          idx < *nk)
        scales[idx] = (float)v;
    }
  }
  return LITHO_OK;
}

}  // extern "C"
