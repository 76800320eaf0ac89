// litho_gb300_cli <config.json> <out_dir> [--quiet|--verbose|--debug] [--tcc fp64|split-bf16]
//
// The GB300 counterpart of the reference program litho.cpp (Modules 1-7,
// litho.cpp:1193-1486): reads the same JSON configuration and writes the same
// BIN file set through the C ABI:
//   mskf_r.bin mskf_i.bin tcc_r.bin tcc_i.bin aerial_image_tcc_direct.bin
//   kernels/krn_{i}_{r,i}.bin kernels/kernel_info.txt scales.bin
//   aerial_image_socs_kernel.bin tmpImgp_pad128.bin tmpImgp_full_128.bin fft_meta.txt
// and prints the reference's [TIME] lines.  Differences from the reference's
// substring parser (litho.cpp:1012-1118): this is a real JSON parser; it also
// reads source.dipole / crossQuadrupole / point parameters, source "Import" with
// source.inputFile, and mask.lineSpace.isHorizontal, which the reference parses
// only partly.  Relative input files resolve against <configDir>/../.. as in
// litho.cpp:1075-1077.  PNG previews are not written.
#include <sys/stat.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "litho_gb300.h"

namespace {

struct J {  // minimal JSON value
  enum T { NUL, NUM, STR, BOOL, OBJ, ARR } t = NUL;
  double num = 0;
  bool b = false;
  std::string str;
  std::map<std::string, J> obj;
  std::vector<J> arr;
  const J* get(const char* k) const {
    if (t != OBJ) return nullptr;
    auto it = obj.find(k);
    return it == obj.end() ? nullptr : &it->second;
  }
};

struct Parser {
  const char* p;
  void ws() {
    while (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t') ++p;
  }
  bool parse(J& v) {
    ws();
    if (*p == '{') {
      ++p;
      v.t = J::OBJ;
      ws();
      if (*p == '}') return ++p, true;
      while (true) {
        ws();
        J key;
        if (*p != '"' || !parse(key)) return false;
        ws();
        if (*p != ':') return false;
        ++p;
        if (!parse(v.obj[key.str])) return false;
        ws();
        if (*p == ',') {
          ++p;
          continue;
        }
        if (*p == '}') return ++p, true;
        return false;
      }
    }
    if (*p == '[') {
      ++p;
      v.t = J::ARR;
      ws();
      if (*p == ']') return ++p, true;
      while (true) {
        v.arr.emplace_back();
        if (!parse(v.arr.back())) return false;
        ws();
        if (*p == ',') {
          ++p;
          continue;
        }
        if (*p == ']') return ++p, true;
        return false;
      }
    }
    if (*p == '"') {
      ++p;
      v.t = J::STR;
      while (*p && *p != '"') {
        if (*p == '\\' && p[1]) ++p;
        v.str += *p++;
      }
      if (*p != '"') return false;
      return ++p, true;
    }
    if (!strncmp(p, "true", 4)) return v.t = J::BOOL, v.b = true, p += 4, true;
    if (!strncmp(p, "false", 5)) return v.t = J::BOOL, v.b = false, p += 5, true;
    if (!strncmp(p, "null", 4)) return v.t = J::NUL, p += 4, true;
    char* e = nullptr;
    v.num = strtod(p, &e);
    if (e == p) return false;
    v.t = J::NUM;
    p = e;
    return true;
  }
};

double num(const J* root, std::initializer_list<const char*> path, double def) {
  const J* v = root;
  for (const char* k : path) {
    if (!v) return def;
    v = v->get(k);
  }
  if (!v) return def;
  if (v->t == J::NUM) return v->num;
  if (v->t == J::BOOL) return v->b ? 1.0 : 0.0;
  return def;
}

std::string str(const J* root, std::initializer_list<const char*> path, const std::string& def) {
  const J* v = root;
  for (const char* k : path) {
    if (!v) return def;
    v = v->get(k);
  }
  return (v && v->t == J::STR) ? v->str : def;
}

std::string parent(const std::string& p) {
  const size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string(".") : (s == 0 ? std::string("/") : p.substr(0, s));
}

std::string resolve(const std::string& root, const std::string& f) {
  return (f.empty() || f[0] == '/') ? f : root + "/" + f;
}

int next_pow2(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}

int verbose = 1;
using clk = std::chrono::steady_clock;
long long us_since(clk::time_point t) {
  return std::chrono::duration_cast<std::chrono::microseconds>(clk::now() - t).count();
}

#define CHECK(call)                                                                         \
  do {                                                                                      \
    int rc_ = (call);                                                                       \
    if (rc_ != LITHO_OK) {                                                                  \
      fprintf(stderr, "Error: %s failed: %s %s\n", #call, litho_status_string(rc_),         \
              ctx ? litho_last_error(ctx) : "");                                            \
      return 1;                                                                             \
    }                                                                                       \
  } while (0)

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "Usage: %s <config.json> <output_dir> [--quiet|--verbose|--debug] [--tcc fp64|split-bf16]\n",
            argv[0]);
    return 1;
  }
  const std::string cfgPath = argv[1], out = argv[2];
  int tccPrec = LITHO_TCC_FP64;
  for (int i = 3; i < argc; ++i) {
    if (!strcmp(argv[i], "--quiet")) verbose = 0;
    else if (!strcmp(argv[i], "--verbose")) verbose = 1;
    else if (!strcmp(argv[i], "--debug")) verbose = 2;
    else if (!strcmp(argv[i], "--tcc") && i + 1 < argc) tccPrec = !strcmp(argv[++i], "split-bf16") ? 1 : 0;
  }
  litho_ctx* ctx = nullptr;
  std::string text;
  {
    FILE* f = fopen(cfgPath.c_str(), "rb");
    if (!f) {
      fprintf(stderr, "Error: Cannot open config file: %s\n", cfgPath.c_str());
      return 1;
    }
    char buf[65536];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    fclose(f);
  }
  J cfg;
  Parser ps{text.c_str()};
  if (!ps.parse(cfg) || cfg.t != J::OBJ) {
    fprintf(stderr, "Error: invalid JSON in %s\n", cfgPath.c_str());
    return 1;
  }
  const std::string projectRoot = parent(parent(parent(cfgPath)));
  const int Lx = (int)num(&cfg, {"mask", "period", "Lx"}, 0), Ly = (int)num(&cfg, {"mask", "period", "Ly"}, 0);
  const int mX = (int)num(&cfg, {"mask", "size", "maskSizeX"}, 0), mY = (int)num(&cfg, {"mask", "size", "maskSizeY"}, 0);
  if (Lx <= 0 || Ly <= 0 || mX <= 0 || mY <= 0) {
    fprintf(stderr, "Error: Invalid mask parameters\n");
    return 1;
  }
  const int S = (int)num(&cfg, {"source", "gridSize"}, 0);
  const float NA = (float)num(&cfg, {"optics", "NA"}, 0), lambda = (float)num(&cfg, {"optics", "wavelength"}, 193);
  const float defocus = (float)num(&cfg, {"optics", "defocus"}, 0);
  const int nkReq = (int)num(&cfg, {"kernel", "count"}, 0);
  CHECK(litho_ctx_create(0, &ctx));
  mkdir(out.c_str(), 0755);
  mkdir((out + "/kernels").c_str(), 0755);
  const auto t_all = clk::now();

  // Module 1: source
  auto t = clk::now();
  std::vector<float> src((size_t)S * S, 0.f);
  const std::string stype = str(&cfg, {"source", "type"}, "");
  if (stype == "Annular") {
    const float p[2] = {(float)num(&cfg, {"source", "annular", "innerRadius"}, 0),
                        (float)num(&cfg, {"source", "annular", "outerRadius"}, 0)};
    CHECK(litho_create_source(src.data(), S, LITHO_SRC_ANNULAR, p, 1));
  } else if (stype == "Dipole") {
    const float p[3] = {(float)num(&cfg, {"source", "dipole", "radius"}, 0),
                        (float)num(&cfg, {"source", "dipole", "offset"}, 0),
                        (float)num(&cfg, {"source", "dipole", "onXAxis"}, 1)};
    CHECK(litho_create_source(src.data(), S, LITHO_SRC_DIPOLE, p, 1));
  } else if (stype == "CrossQuadrupole") {
    const float p[2] = {(float)num(&cfg, {"source", "crossQuadrupole", "radius"}, 0),
                        (float)num(&cfg, {"source", "crossQuadrupole", "offset"}, 0)};
    CHECK(litho_create_source(src.data(), S, LITHO_SRC_CROSS_QUADRUPOLE, p, 1));
  } else if (stype == "Point") {
    const float p[2] = {(float)num(&cfg, {"source", "point", "x"}, 0), (float)num(&cfg, {"source", "point", "y"}, 0)};
    CHECK(litho_create_source(src.data(), S, LITHO_SRC_POINT, p, 1));
  } else if (stype == "Import") {
    CHECK(litho_read_bin(resolve(projectRoot, str(&cfg, {"source", "inputFile"}, "")).c_str(), src.data(),
                         (long long)S * S));
    CHECK(litho_normalize_source(src.data(), S));
  } else {
    fprintf(stderr, "Error: unknown source type '%s'\n", stype.c_str());
    return 1;
  }
  if (verbose) printf("[TIME] Source creation: %lld us\n", us_since(t));

  // Module 2: mask
  t = clk::now();
  std::vector<float> in((size_t)mX * mY, 0.f), msk((size_t)Lx * Ly, 0.f);
  const std::string mtype = str(&cfg, {"mask", "type"}, "");
  if (mtype == "LineSpace") {
    CHECK(litho_create_linespace(in.data(), mX, mY, (int)num(&cfg, {"mask", "lineSpace", "lineWidth"}, 0),
                                 (int)num(&cfg, {"mask", "lineSpace", "spaceWidth"}, 0),
                                 (int)num(&cfg, {"mask", "lineSpace", "isHorizontal"}, 0)));
  } else if (mtype == "Import") {
    CHECK(litho_read_bin(resolve(projectRoot, str(&cfg, {"mask", "inputFile"}, "")).c_str(), in.data(),
                         (long long)mX * mY));
  }
  CHECK(litho_place_mask(in.data(), mX, mY, (float)num(&cfg, {"mask", "dose"}, 1.0), msk.data(), Lx, Ly));
  if (verbose) printf("[TIME] Mask creation: %lld us\n", us_since(t));

  // optics (litho.cpp:1297-1302)
  const float sigma = litho_outer_sigma(src.data(), S);
  const int Nx = litho_optics_n(NA, Lx, sigma, lambda), Ny = litho_optics_n(NA, Ly, sigma, lambda);
  const int tccSize = (2 * Nx + 1) * (2 * Ny + 1);
  const int Fx = next_pow2(Lx), Fy = next_pow2(Ly);
  {
    FILE* f = fopen((out + "/fft_meta.txt").c_str(), "w");  // litho.cpp:1165-1187 (same keys and values)
    if (f) {
      fprintf(f, "physical_size_x %d\nphysical_size_y %d\nfft_size_x %d\nfft_size_y %d\nNx %d\nNy %d\n", Lx, Ly, Fx,
              Fy, Nx, Ny);
      fprintf(f, "conv_size_x %d\nconv_size_y %d\nfft_conv_size_x %d\nfft_conv_size_y %d\n", 4 * Nx + 1, 4 * Ny + 1,
              next_pow2(4 * Nx + 1), next_pow2(4 * Ny + 1));
      fclose(f);
    }
  }
  if (verbose) printf("[PARAM] Outer Sigma: %g  Nx: %d, Ny: %d  TCC Size: %d x %d\n", sigma, Nx, Ny, tccSize, tccSize);

  // Module 3: mask spectrum
  t = clk::now();
  std::vector<float> mr((size_t)Fx * Fy), mi((size_t)Fx * Fy);
  CHECK(litho_fft_mask(ctx, msk.data(), Lx, Ly, mr.data(), mi.data(), LITHO_MEM_HOST));
  if (verbose) printf("[TIME] FFT Mask: %lld us\n", us_since(t));
  CHECK(litho_write_bin((out + "/mskf_r.bin").c_str(), mr.data(), (long long)mr.size()));
  CHECK(litho_write_bin((out + "/mskf_i.bin").c_str(), mi.data(), (long long)mi.size()));

  // Module 4: TCC
  t = clk::now();
  std::vector<double> tcc((size_t)2 * tccSize * tccSize);
  CHECK(litho_calc_tcc(ctx, src.data(), S, sigma, lambda, NA, defocus, Lx, Ly, Nx, Ny, tcc.data(), tccPrec,
                       LITHO_MEM_HOST));
  if (verbose) printf("[TIME] TCC computation: %lld us\n", us_since(t));
  {
    std::vector<float> tr((size_t)tccSize * tccSize), ti((size_t)tccSize * tccSize);
    for (size_t i = 0; i < tr.size(); ++i) {
      tr[i] = (float)tcc[2 * i];
      ti[i] = (float)tcc[2 * i + 1];
    }
    CHECK(litho_write_bin((out + "/tcc_r.bin").c_str(), tr.data(), (long long)tr.size()));
    CHECK(litho_write_bin((out + "/tcc_i.bin").c_str(), ti.data(), (long long)ti.size()));
  }

  // Module 5: TCC-direct image
  t = clk::now();
  std::vector<float> img((size_t)Lx * Ly);
  CHECK(litho_calc_image(ctx, mr.data(), mi.data(), Fx, Fy, tcc.data(), tccSize, Nx, Ny, Lx, Ly, img.data(),
                         LITHO_MEM_HOST));
  if (verbose) printf("[TIME] TCC Image: %lld us\n", us_since(t));
  CHECK(litho_write_bin((out + "/aerial_image_tcc_direct.bin").c_str(), img.data(), (long long)img.size()));

  // Module 6: kernels
  t = clk::now();
  const int nk = nkReq < tccSize ? nkReq : tccSize;
  if (nk < 1) {
    fprintf(stderr, "Error: kernel.count must be >= 1\n");
    return 1;
  }
  std::vector<float> kr((size_t)nk * tccSize), ki((size_t)nk * tccSize), sc(nk);
  CHECK(litho_calc_kernels(ctx, tcc.data(), tccSize, nk, kr.data(), ki.data(), sc.data(), nullptr, nullptr,
                           LITHO_MEM_HOST));
  if (verbose) printf("[TIME] Kernel extraction: %lld us\n", us_since(t));
  CHECK(litho_write_kernel_info((out + "/kernels/kernel_info.txt").c_str(), 2 * Nx + 1, 2 * Ny + 1, nk, sc.data()));
  for (int k = 0; k < nk; ++k) {
    CHECK(litho_write_bin((out + "/kernels/krn_" + std::to_string(k) + "_r.bin").c_str(), kr.data() + (size_t)k * tccSize,
                          tccSize));
    CHECK(litho_write_bin((out + "/kernels/krn_" + std::to_string(k) + "_i.bin").c_str(), ki.data() + (size_t)k * tccSize,
                          tccSize));
  }
  CHECK(litho_write_bin((out + "/scales.bin").c_str(), sc.data(), nk));

  // Module 7: SOCS image on litho.cpp's 128^2 conv grid, with the tmpImgp dumps
  t = clk::now();
  std::vector<float> tmp((size_t)128 * 128);
  CHECK(litho_calc_socs(ctx, mr.data(), mi.data(), Fx, Fy, kr.data(), ki.data(), sc.data(), nk, Nx, Ny, Lx, Ly,
                        img.data(), tmp.data(), 128, LITHO_MEM_HOST));
  if (verbose) printf("[TIME] SOCS Image: %lld us\n", us_since(t));
  CHECK(litho_write_bin((out + "/aerial_image_socs_kernel.bin").c_str(), img.data(), (long long)img.size()));
  {
    const int cx = 4 * Nx + 1, cy = 4 * Ny + 1, ox = (128 - cx) / 2, oy = (128 - cy) / 2;  // litho.cpp:950-960
    std::vector<float> c((size_t)cx * cy);
    for (int y = 0; y < cy; ++y)
      for (int x = 0; x < cx; ++x) c[(size_t)y * cx + x] = tmp[(size_t)(oy + y) * 128 + ox + x];
    CHECK(litho_write_bin((out + "/tmpImgp_pad128.bin").c_str(), c.data(), (long long)c.size()));
    CHECK(litho_write_bin((out + "/tmpImgp_full_128.bin").c_str(), tmp.data(), (long long)tmp.size()));
  }
  if (verbose) printf("[TIME] Total: %lld us\n[DONE] Output saved to: %s\n", us_since(t_all), out.c_str());
  litho_ctx_destroy(ctx);
  return 0;
}
