// Shared declarations of the distance-band kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pgld_internal.cuh"

int pgld_band_offsets(pgld_context* h, const double* pos, long long n_snp, double max_dist,
                      long long* off, void* scratch, size_t scratch_bytes, cudaStream_t st);

namespace pgld {

constexpr int kTile = 32;      // SNPs per tile side of the plain band kernel
constexpr int kMaxBins = 64;   // distance bins per call
constexpr int kModeBinned = 0;
constexpr int kModePairs = 1;
constexpr int kModeWindows = 2;

struct BandArgs {
  int n_pops;
  int W[PGLD_MAX_POPS];
  const uint32_t* planes[PGLD_MAX_POPS];
  const uint32_t* valid[PGLD_MAX_POPS];
  const uint32_t* gext[PGLD_MAX_POPS];  // genotype planes of the values 3..8 (or NULL)
  long long n_snp;
  // binned mode: only pairs whose first SNP lies below n_anchor count
  // (<= 0: every SNP is an anchor)
  long long n_anchor;
  const double* pos;
  double max_dist;
  const double* bcoord;  // binning coordinate (NULL: pos)
  const double* bins;
  int n_bins;
  const long long* item_off;  // [n_blocks + 1] tile work list offsets
  long long n_blocks;
  // binned mode
  double* sums;
  int64_t* pair_counts;
  const pgld_term* terms;
  int n_terms;
  int n_stats;
  // pairs mode
  const long long* pair_off;
  int32_t* counts;
  int32_t* nvalid;
  float* stats;
  int32_t* status;  // device error word of the handle
  int nmax;         // largest per-population sample size (32 * max words)
  int stat_mask;    // genotype pairs mode: columns to compute (bit k = column k)
};

// number of anchors of a binned call (every SNP unless n_anchor limits it)
__host__ __device__ __forceinline__ long long anchors_of(const BandArgs& a) {
  return (a.n_anchor > 0 && a.n_anchor < a.n_snp) ? a.n_anchor : a.n_snp;
}

// tile work list of `tile`-SNP blocks: items[b] = tiles of row block b, then
// exclusively scanned in place (items[n_blocks] = total)
int band_schedule(pgld_context* h, const double* pos, long long n_snp, double max_dist,
                  long long* items, void* scratch, size_t scratch_bytes, cudaStream_t st,
                  int tile = kTile, int col_tile = 0);
int launch_band_plain(pgld_context* h, const BandArgs& a, int mode, cudaStream_t st);
// the one/two-population kernel with the float32 epilogue (pgld_band_fast.cu)
bool band_fast_applies(const BandArgs& a, int mode);
int launch_band_fast(pgld_context* h, const BandArgs& a, int mode, cudaStream_t st);

}  // namespace pgld
