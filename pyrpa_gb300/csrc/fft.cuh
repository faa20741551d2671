// Batched 4-D complex FFT over the (x, y, z, t) grid of the FLEX engine.
//
// The reference transforms each orbital-pair array with one serial FFTW/
// pocketfft call on the CPU (libs/src/fmod.f90:67-116, fft_wrapper.cpp:32-87).
// Here a transform is a short sequence of "axis passes": each pass reads a
// tile of lines into shared memory (coalesced along the fastest index),
// runs a mixed-radix Stockham FFT (radices 8,4,2,3,5,7 and a table-driven
// generic radix for other primes <= 64) and writes the tile back in place.
// Lines of length L = A*B with A, B in {2,3,4,5,8} (L <= 64) use a two-level
// register kernel: one coalesced read with a radix-A DFT in registers, one
// shared-memory exchange, a radix-B DFT and one write.  Longer axes are
// split four-step style into two such passes where possible; axes longer
// than kMaxLine that cannot be split that way use two Stockham passes
// (L = L1*L2) with the twiddle multiply fused into the second pass; the
// frequency index of such an axis is then stored digit-transposed, which
// all pointwise kernels handle through the per-axis position tables below.
// With PYRPA_GB_FFT_PLANE=1, meshes with 2 <= nx, ny <= 64 transform x and
// y in one "plane pass" (one (x, y) plane per CTA in shared memory, rows
// padded to nx + 1) instead of two passes.
// With PYRPA_GB_FFT_LONG=1, axes of length L1 * L2 (L1, L2 in {16, 64})
// that would take the two four-step passes take one "long pass" instead: a
// CTA holds a few adjacent lines whole in shared memory, and the frequency
// order (digit-transposed) is the same.
// Forward is exp(-2 pi i jk/L) (FFTW sign -1), backward exp(+...), both
// unnormalized: the callers fold 1/P into their weights.
#pragma once

#include "common.cuh"

namespace pgb {

constexpr int kMaxLine = 1024;
constexpr int kMaxStages = 16;

struct PassDesc {
  int L;               // line length
  long long S;         // element stride along the line
  long long O;         // number of outer blocks (dims above the line)
  int B;               // lines per CTA
  int nst;             // number of Stockham stages
  int radix[kMaxStages];
  int tw_L1;           // four-step: modulus of the k1 digit (0: no twiddle)
  int tw_Lfull;        // four-step: full axis length
  int tw_post;         // 0: multiply before the line DFT, 1: after
  const double2* tw_line;  // exp(-2 pi i t / L), t < L
  const double2* tw_full;  // exp(-2 pi i t / Lfull), t < Lfull
  const float2* tw_line_f; // the same tables rounded to FP32 for the FP32 kernels
  const float2* tw_full_f; //   (FP64->FP32 conversions run on the FP64 pipe)
  const cdf* tw_line_d;    // and as double-float pairs for the double-float kernels
  const cdf* tw_full_d;
  int fa, fb;              // L = fa * fb for the two-level register kernel (0: Stockham kernel)
  // plane pass: the x (length L) and y (length ny) axes of each (x, y) plane
  // in one kernel; O = number of planes
  int plane;
  int ny;
  int nst_y;
  int radix_y[kMaxStages];
  const double2* tw_line_y;
  const float2* tw_line_y_f;
  const cdf* tw_line_y_d;
  // long pass: a four-step axis of length L = lp_L1 * lp_L2 in one kernel
  // (B lines per CTA, tw_line* for lp_L1, tw_line_y* for lp_L2, tw_full* for L)
  int lp;
  int lp_L1, lp_L2;
  // x-y plane pass: both axes of each square (x, y) plane of side L = fa fb
  // in one kernel (fft_xy_kernel); O = number of planes
  int xy;
  // strided two-level pass staged by TMA (fft2_tma_kernel): tiles of
  // kTmaLines adjacent lines, S a multiple of kTmaLines
  int tma;
};

// Per-axis overrides of the plan's heuristics; 0 keeps the heuristic.
// L1: the first length of a four-step split (axes > 64 without a direct
// two-level kernel); lines: lines per CTA of every pass of the axis.
struct AxisTune {
  int L1 = 0;
  int lines = 0;
};
struct PlanTune {
  AxisTune ax[4];
};

// The settings an autotuner may try for one axis of length n with
// elem-byte elements: the heuristic first, then every four-step split whose
// two lengths have a two-level kernel, each with 8, 16, 32 or 64 lines per
// CTA where the pass's shared memory fits its launch.
std::vector<AxisTune> fft_axis_candidates(int n, int elem_bytes);

// Position tables of one axis: pos[k] is where logical index k is stored,
// rev[p] the position of logical -k for the value stored at position p.
struct AxisMap {
  int n = 1;
  std::vector<int> pos, rev, logical;
};

class FFT4D {
 public:
  FFT4D() = default;
  // tune: per-axis overrides (null: the heuristics)
  FFT4D(int nx, int ny, int nz, int nt, int elem_bytes, const PlanTune* tune = nullptr);
  // frees the device position tables (plans made for timing only)
  void release_tables();
  long long P() const { return P_; }
  const int* dims() const { return dims_; }
  // in-place transform of nb arrays stored back to back (stride P)
  template <typename R> void forward(cx<R>* data, int nb, cudaStream_t s) const;
  template <typename R> void backward(cx<R>* data, int nb, cudaStream_t s) const;
  // spatial-only (x,y,z) forward transform; the t axis is left untouched
  template <typename R> void forward_space(cx<R>* data, int nb, cudaStream_t s) const;
  // its inverse (unnormalized): spatial axes from the forward_space layout back to natural order
  template <typename R> void backward_space(cx<R>* data, int nb, cudaStream_t s) const;
  const AxisMap& axis(int a) const { return maps_[a]; }
  // device copies of the position tables (pos, rev, logical) of each axis
  const int* d_pos(int a) const { return d_tables_ + off_pos_[a]; }
  const int* d_rev(int a) const { return d_tables_ + off_rev_[a]; }
  const int* d_logical(int a) const { return d_tables_ + off_log_[a]; }

 private:
  int dims_[4] = {1, 1, 1, 1};
  long long P_ = 1;
  std::vector<PassDesc> fwd_, bwd_, fwd_space_, bwd_space_;
  AxisMap maps_[4];
  int* d_tables_ = nullptr;
  int off_pos_[4] = {0, 0, 0, 0}, off_rev_[4] = {0, 0, 0, 0}, off_log_[4] = {0, 0, 0, 0};
  template <typename R> void run(const std::vector<PassDesc>& passes, cx<R>* data, int nb,
                                 int sign, cudaStream_t s) const;
};

// Cached FFT plan for a grid (plans and twiddle tables live for the process).
// With PYRPA_GB_FFT_TUNE=1 a new plan's per-axis settings are chosen by
// timing the candidates of fft_axis_candidates on a scratch array (one axis
// at a time, the others fixed at their best so far).
const FFT4D& fft_plan(int nx, int ny, int nz, int nt, int elem_bytes);

// Optional live timing of every FFT pass launch with CUDA events on the
// launching stream: launches, summed milliseconds and algorithmic bytes
// (each element read once and written once per pass).
void fft_profile_enable(bool on);
void fft_profile_collect(double* launches, double* ms, double* bytes);

}  // namespace pgb
