// litho_gb300_hls.hpp -- C++-linkage shims with the signatures of the
// reference's FPGA top functions, backed by the GB300 library, so code written
// against those tops (e.g. the reference's C-simulation testbenches) runs on
// the GPU unchanged.
//
// * calc_socs_2048_hls_stream_refactored_v18 replaces
//   source/SOCS_HLS/src/socs_2048_stream_refactored_v18_hls_fft.h:86-97:
//   mskf planes (Ly x Lx, DC at (Ly/2, Lx/2)), nk kernels k-major
//   ((2ny+1)(2nx+1) each), scales; writes the 128 x 128 fftshifted intensity
//   before Fourier interpolation (litho.cpp's tmpImgp_full_128) to both
//   tmpImg_ddr and output.
// * calc_tcc replaces source/TCC_HLS/hls/src/calc_tcc.h:78-86 with the
//   OpticalParams layout of source/TCC_HLS/hls/src/data_types.h; sh and oSgm are
//   taken from the caller as there.
//
// Both use a process-wide context on the current CUDA device and block until
// their outputs are written.  On failure (no GPU, bad sizes) the outputs are
// filled with NaN, since these void functions have no status to return.
#ifndef LITHO_GB300_HLS_HPP
#define LITHO_GB300_HLS_HPP

#include <complex>

typedef float data_t;
typedef std::complex<data_t> cmpxData_t;

struct OpticalParams {
  data_t NA;
  data_t lambda;
  data_t defocus;
  data_t Lx;
  data_t Ly;
  data_t outerSigma;
  int srcSize;
  int Nx;
  int Ny;
};

void calc_socs_2048_hls_stream_refactored_v18(float* mskf_r, float* mskf_i, float* krn_r, float* krn_i,
                                              float* scales, float* tmpImg_ddr, float* output, int nk,
                                              int nx_actual, int ny_actual, int Lx, int Ly);

void calc_tcc(data_t* src, int srcSize, cmpxData_t* tcc, OpticalParams& params, int tccSize, int sh, int oSgm);

#endif  // LITHO_GB300_HLS_HPP
