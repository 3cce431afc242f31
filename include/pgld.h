/*
 * pgld.h -- C ABI of libpgld, the GB300 (sm_103a) two-locus LD library.
 *
 * Plain pointers and sizes only.  Every entry point returns an int status
 * (PGLD_OK == 0, negative on error), never throws and never aborts; the
 * message for the last failure is available from pgld_last_error().
 * Buffers are owned by the caller: device buffers are passed as raw device
 * pointers, and work is enqueued on the given stream (a cudaStream_t passed
 * as void*, NULL = legacy default stream).  Calls are asynchronous unless
 * noted ("synchronises"), i.e. where a size must come back to the host.
 * The library owns only the handle and its device workspace; distinct
 * handles may be used from distinct host threads.
 *
 * Reference interfaces cited below are files of kr-colab/pg_gpu.
 */
#ifndef PGLD_H
#define PGLD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PGLD_OK 0
#define PGLD_ERR_INVALID_ARG (-1)
#define PGLD_ERR_CUDA (-2)
#define PGLD_ERR_TOO_LARGE (-3)
#define PGLD_ERR_UNSUPPORTED (-4)
#define PGLD_ERR_TIMEOUT (-5)
#define PGLD_ERR_NO_MEMORY (-6)

#define PGLD_MAX_POPS 4

/* Output element types. */
#define PGLD_F64 0
#define PGLD_F32 1

/* Count-kernel forms. */
#define PGLD_FORM_PLAIN 0 /* bit-packed AND + popcount                  */
#define PGLD_FORM_TC 1    /* tcgen05 tensor-core contraction (sm_103a)  */

typedef struct pgld_context* pgld_handle;

/* ----------------------------------------------------------------------
 * Per-population bit planes of a haplotype panel.
 *
 * For population p with H_p haplotypes, n_words[p] = ceil(H_p / 32) and
 * planes[p] holds, for every SNP s, 2 * n_words[p] uint32 words:
 * words [0, n_words) are the carrier plane (bit h set iff hap[h][s] == 1)
 * and words [n_words, 2 n_words) the reference plane (hap[h][s] == 0).
 * valid[p] is optional ([n_snp][n_words] bits of hap >= 0); it is needed
 * only when the panel holds values other than -1/0/1 AND missing data, in
 * which case the pairwise-valid n is not n11+n10+n01+n00.  When valid[p]
 * is NULL the per-pair n of population p is n11+n10+n01+n00, which is the
 * reference's n_valid for 0/1/-1 data (ld_pipeline.py:158-172).
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t n_pops;
  int32_t n_words[PGLD_MAX_POPS];
  const uint32_t* planes[PGLD_MAX_POPS];
  const uint32_t* valid[PGLD_MAX_POPS];
  int64_t n_snp;
} pgld_hap_panel;

/* Handle management. */
int pgld_version(void);
int pgld_create(int device, pgld_handle* out);
int pgld_destroy(pgld_handle h);
/* Message of the last failed call on h (h may be NULL: last failure of any
 * call on this host thread).  Valid until the next call on the thread. */
const char* pgld_last_error(pgld_handle h);
/* Reads and clears the device-side error word of h (synchronises).  0: no
 * error.  Kernels record the first failure of a launch and skip the rest of
 * its work: 2001 / 3001 corrupt tile work list; 3002 - 3005 a bounded
 * mbarrier wait of a tensor-core kernel expired (TMA producer, MMA issuer,
 * epilogue) -- the launch drained its copies and MMAs, freed its tensor
 * memory and returned, and the handle stays usable (PGLD_DEVICE_WAIT_EXPIRED
 * tells these codes apart); 3100 - 3102 a window or SNP index outside its
 * panel. */
int pgld_device_status(pgld_handle h, int32_t* code_out, void* stream);
#define PGLD_DEVICE_WAIT_EXPIRED(code) ((code) >= 3002 && (code) <= 3005)

/* Test hook (no counterpart in the reference): kind PGLD_TEST_FAULT_NO_COPIES
 * makes the next tensor-core band launch on h issue no operand copies and
 * shortens its bounded waits to ~10 ms, so that the MMA issuer's wait for
 * the first stage expires and the launch ends through its error path (a
 * wait-expiry code in the device status word).  The hook faults and hangs
 * nothing; it is cleared by that launch.  kind 0 clears it. */
#define PGLD_TEST_FAULT_NO_COPIES 1
int pgld_set_test_fault(pgld_handle h, int32_t kind);

/* Pack rows of an int8 (n_rows_total x n_snp) haplotype matrix (row stride
 * ld bytes, values 1 / 0 / -1) into the bit planes above.  rows: device
 * int32 row indices (NULL = rows 0..n_rows-1).  valid may be NULL.
 * flags: device int32[2], OR-ed: flags[0] |= 1 if a -1 was seen,
 * flags[1] |= 1 if a value outside {-1,0,1} was seen.
 * Replaces the per-call gathers of ld_pipeline.compute_counts_for_pairs
 * (ld_pipeline.py:150-158) and HaplotypeMatrix.tally_gpu_haplotypes
 * (haplotype_matrix.py:1344-1349). */
int pgld_pack_haplotypes(pgld_handle h, const int8_t* hap, int64_t ld, int64_t n_snp,
                         const int32_t* rows, int32_t n_rows, uint32_t* planes,
                         uint32_t* valid, int32_t* flags, void* stream);

/* Joint counts [n11, n10, n01, n00] of listed SNP pairs for one
 * population; counts row stride counts_ld (int32 elements, >= 4).
 * n_valid (nullable) receives the pairwise-valid n.
 * Replaces ld_pipeline.compute_counts_for_pairs (ld_pipeline.py:130-175). */
int pgld_hap_counts_pairs(pgld_handle h, const uint32_t* planes, const uint32_t* valid,
                          int32_t n_words, int64_t n_snp, const int32_t* idx_i,
                          const int32_t* idx_j, int64_t n_pairs, int32_t* counts,
                          int64_t counts_ld, int32_t* n_valid, void* stream);

/* All-pairs (i<j, row-major upper triangle) counts of one population, the
 * output of HaplotypeMatrix.tally_gpu_haplotypes (haplotype_matrix.py:
 * 1320-1434), correct at any sample size.  n_valid may be NULL. */
int pgld_hap_tally(pgld_handle h, const uint32_t* planes, const uint32_t* valid,
                   int32_t n_words, int64_t n_snp, int32_t* counts, int32_t* n_valid,
                   void* stream);

/* ----------------------------------------------------------------------
 * Statistic terms.  A statistic column is the weighted sum of terms; each
 * term is one case formula of the reference evaluated on populations
 * pops[0..3] (roles per kind below).  Numerators and denominators are
 * formed exactly in 64-bit integers and divided once (float64 for
 * PGLD_F64 output, float32 for PGLD_F32).
 * ---------------------------------------------------------------------- */
enum pgld_kind {
  PGLD_DD_II = 0,      /* dd(i,i)            ld_statistics.py:1116-1128 */
  PGLD_DD_IJ = 1,      /* dd(i,j)            ld_statistics.py:1131-1169 */
  PGLD_DZ_III = 2,     /* dz(i,i,i)          ld_statistics.py:1172-1189 */
  PGLD_DZ_IIJ = 3,     /* dz(i,i,j) pops=i,j ld_statistics.py:1212-1225 */
  PGLD_DZ_IJI = 4,     /* dz(i,j,i) pops=i,j ld_statistics.py:1227-1240 */
  PGLD_DZ_IJJ = 5,     /* dz(i,j,j) pops=i,j ld_statistics.py:1242-1253 */
  PGLD_DZ_IJK = 6,     /* dz(i,j,k)          ld_statistics.py:1255-1270 */
  PGLD_PI2_IIII = 7,   /* pi2(i,i,i,i)       ld_statistics.py:1275-1296 */
  PGLD_PI2_TRIPLE = 8, /* pops = triple, single  ld_statistics.py:1415-1445 */
  PGLD_PI2_IIKK = 9,   /* kernel form        haplotype_kernels.py:180-190 */
  PGLD_PI2_IIKK_SYM = 10, /* symmetrised     ld_statistics.py:1327-1339 */
  PGLD_PI2_IIKL = 11,  /* pops = i,k,l       ld_statistics.py:1448-1481 */
  PGLD_PI2_IJKK = 12,  /* pops = i,j,k       ld_statistics.py:1484-1516 */
  PGLD_PI2_IJIJ = 13,  /* pops = i,j         ld_statistics.py:1349-1402 */
  PGLD_PI2_SHARED = 14,/* pops = shared,a,b  ld_statistics.py:1519-1589 */
  PGLD_PI2_ALLDIFF = 15,/* pops = i,j,k,l    ld_statistics.py:1592-1617 */
  PGLD_R = 16,         /* haplotype_kernels.py:20-30, NaN if undefined */
  PGLD_R2 = 17,        /* haplotype_kernels.py:32-42 */
  PGLD_DPRIME = 18,    /* haplotype_kernels.py:44-62 */
  /* Genotype (unphased diploid) kinds on 9-way counts, the cases of
   * compute_all_{dd,dz,pi2}_geno (genotype_kernels.py:560-886). */
  PGLD_G_DD_II = 32,   /* _DD_GENO_SINGLE_KERN   genotype_kernels.py:27-71   */
  PGLD_G_DD_IJ = 33,   /* _DD_GENO_BETWEEN_KERN  genotype_kernels.py:73-83   */
  PGLD_G_DZ_III = 34,  /* _DZ_III_KERN           genotype_kernels.py:235-279 */
  PGLD_G_DZ_IIJ = 35,  /* _DZ_IIJ_KERN pops=i,j  genotype_kernels.py:208-215 */
  PGLD_G_DZ_IJI = 36,  /* _DZ_IJI_KERN pops=i,j  genotype_kernels.py:217-224 */
  PGLD_G_DZ_IJJ = 37,  /* _DZ_IJJ_KERN pops=i,j  genotype_kernels.py:226-233 */
  PGLD_G_DZ_IJK = 38,  /* _DZ_DISTINCT_KERN      genotype_kernels.py:199-206 */
  PGLD_G_PI2_IIII = 39,/* _PI2_IIII_KERN         genotype_kernels.py:364-398 */
  PGLD_G_PI2_IIIJ = 40,/* pops=triple,single, calls (t,t,..) genotype_kernels.py:319-329 */
  PGLD_G_PI2_IJII = 41,/* pops=triple,single, other calls    genotype_kernels.py:330-339 */
  PGLD_G_PI2_IIKK = 42,/* genotype_kernels.py:286-291 */
  PGLD_G_PI2_IIKL = 43,/* pops=i,k,l genotype_kernels.py:293-299 */
  PGLD_G_PI2_IJKK = 44,/* pops=i,j,k genotype_kernels.py:301-307 */
  PGLD_G_PI2_IJIJ = 45,/* pops=i,j   genotype_kernels.py:341-361 */
  PGLD_G_PI2_SHARED = 46,/* pops=shared,a,b genotype_kernels.py:309-317 */
  PGLD_G_PI2_ALLDIFF = 47,/* genotype_kernels.py:279-285 */
  PGLD_G_SIGMA_D2 = 48,/* DD/pi2 ratio, NaN if undefined  genotype_kernels.py:91-169 */
  PGLD_G_RH_R = 49,    /* Rogers-Huff r (pairwise-complete), ld_statistics.py:410-443 */
  PGLD_G_RH_R2 = 50    /* Rogers-Huff r^2 */
};

typedef struct {
  int32_t stat;    /* output column */
  int32_t kind;    /* enum pgld_kind */
  int32_t pops[4];
  double weight;   /* the column is sum over its terms of weight * value */
} pgld_term;

/* Per-pair counts of up to 4 populations, as device pointers. */
typedef struct {
  int32_t n_pops;
  const int32_t* counts[PGLD_MAX_POPS]; /* [n_pairs][>=4] int32 */
  int64_t counts_ld[PGLD_MAX_POPS];     /* elements between pairs */
  const int32_t* n_valid[PGLD_MAX_POPS];/* NULL: n = n11+n10+n01+n00 */
  int64_t nvalid_ld[PGLD_MAX_POPS];     /* elements between pairs (0 ok) */
} pgld_pair_counts;

/* The moments statistic table of n_pops populations as terms (host only, no
 * device needed): the columns follow moments ld_names order and each term is
 * the case selection of haplotype_kernels.compute_multi_pop_statistics_batch_hap
 * (haplotype_kernels.py:335-640) applied to generate_stat_specs
 * (ld_pipeline.py:388-457).  With out == NULL only the sizes are returned. */
int pgld_stat_terms(int32_t n_pops, pgld_term* out, int32_t capacity, int32_t* n_terms_out,
                    int32_t* n_stats_out);

/* Statistic columns from per-pair counts.  out is [n_pairs][out_ld] of
 * out_dtype.  Replaces ld_statistics.dd/dz/pi2/r/r_squared/d_prime
 * (ld_statistics.py:13-246), compute_two_pop_statistics_batch
 * (ld_pipeline.py:271-322), compute_single_pop_statistics_batch
 * (ld_pipeline.py:330-349) and compute_multi_pop_statistics_batch_hap
 * (haplotype_kernels.py:584-640). */
int pgld_hap_stats(pgld_handle h, const pgld_pair_counts* counts, int64_t n_pairs,
                   const pgld_term* terms, int32_t n_terms, int32_t n_stats, void* out,
                   int32_t out_dtype, int64_t out_ld, void* stream);

/* Number of pairs i<j with pos[j] - pos[i] <= max_dist (synchronises).
 * pos: device float64, sorted ascending.  offsets (nullable, device int64
 * [n_snp + 1]) receives the exclusive prefix sum of the per-anchor pair
 * counts (offsets[n_snp] = total), the quantity the reference's chunker
 * cumulates (ld_pipeline.py:85-101). */
int pgld_count_pairs_within(pgld_handle h, const double* pos, int64_t n_snp,
                            double max_dist, int64_t* n_pairs_out, int64_t* offsets,
                            void* stream);

/* Pairs of the distance band whose first SNP lies in [i_begin, i_end), in
 * the reference's order (i-major, j ascending), written to idx_i / idx_j;
 * n_pairs must equal the number of such pairs (synchronises to check it).
 * One call per chunk of ld_pipeline.iter_pairs_within_distance
 * (ld_pipeline.py:57-122). */
int pgld_pairs_within(pgld_handle h, const double* pos, int64_t n_snp, double max_dist,
                      int64_t i_begin, int64_t i_end, int32_t* idx_i, int32_t* idx_j,
                      int64_t n_pairs, void* stream);

/* Per-pair outputs over the distance band of one population, in the
 * reference's pair order: counts [n_pairs][4] int32, n_valid [n_pairs]
 * (nullable), and stats [n_pairs][4] float32 = r^2, DD, Dz, pi2 (nullable).
 * n_pairs must equal pgld_count_pairs_within's result.  Fuses
 * iter_pairs_within_distance + compute_counts_for_pairs +
 * compute_single_pop_statistics_batch + r_squared. */
int pgld_hap_band_pairs(pgld_handle h, const pgld_hap_panel* panel, const double* pos,
                        double max_dist, int32_t* counts, int32_t* n_valid, float* stats,
                        int64_t n_pairs, int32_t form, void* stream);

/* Distance-binned sums of the moments LD statistics of n_pops (1..4)
 * populations over every pair i<j with pos[j]-pos[i] <= max_dist.
 * The distance used for binning is bin_coord[j]-bin_coord[i] (bin_coord
 * NULL: pos) in its absolute value; bins are right-open, [bins[k],
 * bins[k+1]), digitize semantics.  sums: [n_bins][n_stats] float64
 * (n_stats = 3, 15, 45, 105 in moments ld_names order), overwritten;
 * pair_counts: [n_bins] int64, nullable.  Per-pair statistics are formed
 * in float32 from exact integer numerators; bins accumulate in float64.
 * Replaces moments_ld._compute_ld_sums (moments_ld.py:248-343) and
 * HaplotypeMatrix.compute_ld_statistics_gpu_{single_pop,two_pops}
 * (haplotype_matrix.py:1592-1866). */
int pgld_hap_binned_sums(pgld_handle h, const pgld_hap_panel* panel, const double* pos,
                         double max_dist, const double* bin_coord, const double* bins,
                         int32_t n_bins, double* sums, int64_t* pair_counts, int32_t form,
                         void* stream);

/* pgld_hap_binned_sums over the pairs (i, j) whose first SNP i lies in
 * [anchor_begin, anchor_end) (0 <= anchor_begin <= anchor_end <= n_snp):
 * one rank's share when the anchors are split across devices, each pair
 * computed once.  The kernels read only the SNPs from anchor_begin up to the
 * last partner within max_dist of anchor_end - 1, found on the device
 * (synchronises unless anchor_end == n_snp).  The partition hook of the
 * binned sums; the reference has no multi-device path (its counterpart is
 * the single-device moments_ld._compute_ld_sums, moments_ld.py:248-343). */
int pgld_hap_binned_sums_range(pgld_handle h, const pgld_hap_panel* panel, const double* pos,
                               double max_dist, const double* bin_coord, const double* bins,
                               int32_t n_bins, int64_t anchor_begin, int64_t anchor_end,
                               double* sums, int64_t* pair_counts, int32_t form, void* stream);

/* Dense all-pairs LD of one population (planes: carrier / reference words
 * as above, n_words per plane): D_out[i][j] = pAB - p_i p_j and r2_out[i][j]
 * = D^2 / (p_i (1 - p_i) p_j (1 - p_j)) (0 where that is not positive) with
 * pAB = n11 / n over the pair's valid haplotypes (0 where n = 0) and p per
 * site over its valid haplotypes, each rounded operation by operation as the
 * reference's float64 matrix expressions; zero diagonal; row stride ld
 * (float64 elements); either output may be NULL.  Replaces
 * HaplotypeMatrix._pairwise_ld_core / pairwise_LD_v / pairwise_r2
 * (haplotype_matrix.py:1092-1170) for 0/1/-1 panels. */
int pgld_hap_pairwise_ld(pgld_handle h, const uint32_t* planes, int32_t n_words, int64_t n_snp,
                         double* D_out, double* r2_out, int64_t ld, void* stream);

/* Every pair i < j grouped by distance bin (pos[j] - pos[i] in [bins[b],
 * bins[b + 1]), right-open): its value is the pair's r^2 from the joint
 * counts of planes (ld_statistics.r_squared, NaN where undefined) or, with
 * pair_values non-NULL, pair_values[k] of the condensed upper triangle (k =
 * i (2 n - i - 1) / 2 + j - i - 1); NaN values are skipped.  With values_out
 * NULL the call counts the pairs of each bin into HOST bin_counts
 * (synchronises); with values_out non-NULL (device, sum of bin_counts
 * doubles) it writes the values bin after bin, bin_counts being the counts of
 * the previous call on the same inputs.  The binning of
 * HaplotypeMatrix.windowed_r_squared (haplotype_matrix.py:1282-1296). */
int pgld_pairs_by_bin(pgld_handle h, const uint32_t* planes, int32_t n_words,
                      const double* pair_values, int64_t n_snp, const double* pos,
                      const double* bins, int32_t n_bins, int64_t* bin_counts,
                      double* values_out, void* stream);

/* Order statistics of segments of a device array of non-negative doubles:
 * segment s is values[seg_offsets[s] .. seg_offsets[s + 1]) (HOST offsets,
 * n_seg + 1 of them), targets (HOST int64 pairs) name (segment, rank), and
 * out[t] (HOST) receives the rank-th smallest value (0-based) of the
 * segment, by radix selection on the device (synchronises).  The per-bin
 * percentiles of windowed_r_squared (haplotype_matrix.py:1302-1312) are the
 * linear interpolation of two such order statistics. */
int pgld_segment_kth(pgld_handle h, const double* values, const int64_t* seg_offsets, int32_t n_seg,
                     const int64_t* targets, int32_t n_targets, double* out, void* stream);

/* ----------------------------------------------------------------------
 * Genotype (unphased diploid dosage) path.
 *
 * A population of N individuals is packed into W = ceil(N / 32) words per
 * plane and three planes per SNP: planes[s][0:W] = (g == 0),
 * [W:2W] = (g == 1), [2W:3W] = (g == 2).  Missing (-1) is in no plane.
 * valid (optional, [n_snp][W] bits of g >= 0) and ext (optional,
 * [n_snp][6W]: planes of the values 3..8) are needed only when the matrix
 * holds values above 2: the reference's counting kernel counts such an
 * individual as valid and, through its class index 3 g_i + g_j, folds the
 * values 3..8 at the second SNP into the classes 3..8 (ld_pipeline.py:
 * 193-210); ext reproduces that.  Populations hold at most 8,192
 * individuals (the exact 64-bit statistic numerators).
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t n_pops;
  int32_t n_words[PGLD_MAX_POPS];
  const uint32_t* planes[PGLD_MAX_POPS];
  const uint32_t* valid[PGLD_MAX_POPS];
  const uint32_t* ext[PGLD_MAX_POPS];
  int64_t n_snp;
} pgld_geno_panel;

/* Pack rows of an int8 (n_rows_total x n_snp) dosage matrix (row stride ld
 * bytes, values 0/1/2, negative = missing) into the planes above (valid and
 * ext nullable).  flags:
 * device int32[2], flags[0] |= 1 if a negative value was seen (the
 * reference's has_missing, ld_pipeline.py:253), flags[1] |= 1 if a value
 * above 2 was seen.  Replaces the gathers of
 * ld_pipeline.compute_genotype_counts_for_pairs (ld_pipeline.py:242-250). */
int pgld_pack_genotypes(pgld_handle h, const int8_t* geno, int64_t ld, int64_t n_snp,
                        const int32_t* rows, int32_t n_rows, uint32_t* planes, uint32_t* valid,
                        uint32_t* ext, int32_t* flags, void* stream);

/* 9-way counts [n00, n01, n02, n10, ..., n22] (row stride counts_ld >= 9)
 * of listed SNP pairs and the pairwise-valid n (nullable).  Replaces
 * ld_pipeline.compute_genotype_counts_for_pairs + _GENO_COUNTS_KERN
 * (ld_pipeline.py:183-263). */
int pgld_geno_counts_pairs(pgld_handle h, const uint32_t* planes, const uint32_t* valid,
                           const uint32_t* ext, int32_t n_words, int64_t n_snp, const int32_t* idx_i,
                           const int32_t* idx_j, int64_t n_pairs, int32_t* counts,
                           int64_t counts_ld, int32_t* n_valid, void* stream);

/* The moments statistic table of n_pops populations as genotype terms (host
 * only): the case selection of compute_multi_pop_statistics_batch_geno
 * (genotype_kernels.py:889-936) applied to generate_stat_specs
 * (ld_pipeline.py:388-457). */
int pgld_geno_stat_terms(int32_t n_pops, pgld_term* out, int32_t capacity, int32_t* n_terms_out,
                         int32_t* n_stats_out);

/* Statistic columns from per-pair 9-way counts (counts_ld >= 9), genotype
 * kinds only.  Replaces compute_multi_pop_statistics_batch_geno
 * (genotype_kernels.py:889-936), ld_statistics_genotype.sigma_d2_geno
 * (ld_statistics_genotype.py:1518-1598) and the per-pair Rogers-Huff r. */
int pgld_geno_stats(pgld_handle h, const pgld_pair_counts* counts, int64_t n_pairs,
                    const pgld_term* terms, int32_t n_terms, int32_t n_stats, void* out,
                    int32_t out_dtype, int64_t out_ld, void* stream);

/* Per-pair outputs over the distance band of one population, in the
 * reference's pair order: counts [n_pairs][9] int32 (nullable), n_valid
 * (nullable) and stats [n_pairs][4] float32 = Rogers-Huff r^2 (pairwise-
 * complete), DD, Dz, pi2 (nullable; 16-byte aligned), of which only the
 * columns in stat_mask (bit k = column k) are evaluated, the others written
 * as 0.  n_pairs must equal pgld_count_pairs_within's result.  form
 * PGLD_FORM_TC counts on the tensor cores (dosages 0/1/2 and missing only:
 * no valid / ext planes), PGLD_FORM_PLAIN with AND + popcount.  Fuses
 * iter_pairs_within_distance + compute_genotype_counts_for_pairs + the
 * single-population genotype statistics + rogers_huff_r_squared. */
int pgld_geno_band_pairs(pgld_handle h, const pgld_geno_panel* panel, const double* pos,
                         double max_dist, int32_t* counts, int32_t* n_valid, float* stats,
                         int32_t stat_mask, int64_t n_pairs, int32_t form, void* stream);

/* Distance-binned sums of the moments genotype statistics of n_pops (1..4)
 * populations, arguments and bins as pgld_hap_binned_sums.  Replaces
 * moments_ld._compute_ld_sums with use_genotypes=True (moments_ld.py:248-343). */
int pgld_geno_binned_sums(pgld_handle h, const pgld_geno_panel* panel, const double* pos,
                          double max_dist, const double* bin_coord, const double* bins,
                          int32_t n_bins, double* sums, int64_t* pair_counts, void* stream);
/* The same sums with a choice of form: PGLD_FORM_PLAIN (pgld_geno_binned_sums)
 * or PGLD_FORM_TC, the moments of each population's pairs from tcgen05 MMAs
 * (dosages 0..2 and missing only: no ext planes) and the same exact-integer
 * term table per pair, summed per bin in float32 warp partials and float64
 * slots. */
int pgld_geno_binned_sums_form(pgld_handle h, const pgld_geno_panel* panel, const double* pos,
                               double max_dist, const double* bin_coord, const double* bins,
                               int32_t n_bins, double* sums, int64_t* pair_counts, int32_t form,
                               void* stream);

/* Per-window sums over batched, uneven windows in one launch, one
 * population.  Window w holds the SNPs snp_idx[win_begin[w] .. win_end[w])
 * (device int64 bounds; device int32 indices into the panel, n_idx entries;
 * snp_idx NULL = the identity with n_idx = n_snp); windows may overlap and
 * every pair a < b inside a window contributes.  sums:
 * [n_win][6] float64 = r^2 (pairs where it is defined), sigma_D^2 = DD / pi2
 * numerators (pairs with n >= 4; 0 where the pi2 numerator is 0), DD, Dz,
 * pi2 (single-population moments statistics; 0 below n = 4), naive r^2 of
 * per-site allele frequencies.  counts: [n_win][3] int64 = pairs, pairs with
 * r^2 defined, pairs with n >= 4.  form PGLD_FORM_TC counts on the tensor
 * cores (<= 2048 haplotypes, no validity plane), PGLD_FORM_PLAIN with AND +
 * popcount.  Replaces the per-window loops of
 * _zns_from_precomputed / _zns_tiled over _tile_counts / _tile_sigma_d2 /
 * _tile_r2_naive (ld_statistics.py:281-341, 534-676).  Synchronises. */
int pgld_hap_window_sums(pgld_handle h, const pgld_hap_panel* panel, const int32_t* snp_idx,
                         int64_t n_idx, const int64_t* win_begin, const int64_t* win_end,
                         int32_t n_win, double* sums, int64_t* counts, int32_t form,
                         void* stream);

/* Per-SNP row and column sums of one window statistic, for Kim and Nielsen's
 * omega over batched windows (one launch).  Windows as pgld_hap_window_sums
 * (they may overlap).  For every pair of list positions a < b of window w
 * (a, b relative to win_begin[w]), the pair's value of column stat (0..5 of
 * pgld_hap_window_sums: 1 = sigma_D^2 = DD / pi2 numerators, 5 = naive r^2)
 * is added to row_sums[out_off[w] + a] and col_sums[out_off[w] + b] (float64,
 * n_out entries each, zeroed by the call; out_off device int64, window w
 * owning win_end[w] - win_begin[w] entries).  The prefix sums of these give
 * the within / between block sums of every split point of
 * ld_statistics.omega (ld_statistics.py:761-862) without the m x m matrix.
 * Plain (AND + popcount) counts.  Synchronises. */
int pgld_hap_window_snp_sums(pgld_handle h, const pgld_hap_panel* panel, const int32_t* snp_idx,
                             int64_t n_idx, const int64_t* win_begin, const int64_t* win_end,
                             int32_t n_win, const int64_t* out_off, int32_t stat,
                             double* row_sums, double* col_sums, int64_t n_out, void* stream);

/* locate_unlinked pruning on the host (as the reference's): sliding windows
 * of `size` variants advanced by `step`; within a window, for still-active
 * variants i < j in order, j is dropped when r2 of the pair (i, j) exceeds
 * threshold.  r2: HOST float64 values of the band pairs j - i < size in row
 * order (row i at pair_off[i], pair k of it j = i + 1 + k, as
 * pgld_count_pairs_within / pgld_pairs_within over positions 0..n_snp-1 with
 * max_dist size - 1); pair_off: HOST int64 [n_snp + 1].  loc: HOST uint8
 * [n_snp] out, 1 = kept.  Replaces the pruning loop of
 * HaplotypeMatrix.locate_unlinked (haplotype_matrix.py:1172-1233). */
int pgld_prune_unlinked(pgld_handle h, const double* r2, const int64_t* pair_off, int64_t n_snp,
                        int32_t size, int32_t step, double threshold, uint8_t* loc);

/* VCF GT reading on the host (no device, no handle).  pgld_vcf_scan counts
 * the samples of the #CHROM header line and the data records of a VCF text
 * (already decompressed).  pgld_vcf_parse_gt writes the GT alleles of the
 * selected samples (sample_cols: n_sel column indices into the VCF samples,
 * NULL = all, n_sel = n_samples) as the int8 haplotype matrix of
 * HaplotypeMatrix.from_vcf (haplotype_matrix.py:293-404): row k = first
 * allele of selected sample k, row n_sel + k = its second allele, n_records
 * columns; '.' or an empty allele is -1, a haploid call's second allele -1,
 * allele numbers clipped to 127; pos: int64 [n_records] POS column. */
int pgld_vcf_scan(const char* text, int64_t len, int32_t* n_samples, int64_t* n_records);
int pgld_vcf_parse_gt(const char* text, int64_t len, int32_t n_samples, int64_t n_records,
                      const int32_t* sample_cols, int32_t n_sel, int8_t* hap, int64_t* pos);

/* The GT alleles of a VCF text packed straight into the bit planes of
 * pgld_pack_haplotypes for n_pops populations, with no int8 haplotype matrix
 * (the path HaplotypeMatrix.from_vcf -> load_pop_file -> per-call gathers of
 * haplotype_matrix.py:293-404 and ld_pipeline.py:150-158 takes).  hap_rows:
 * HOST int32 VCF haplotype indices (h < n_samples: first allele of VCF
 * sample h, else the second allele of sample h - n_samples), population p
 * owning hap_rows[pop_offsets[p] .. pop_offsets[p + 1]) in bit order.
 * planes: HOST uint32; population p (W_p = max(1, ceil(n_p / 32)) words)
 * starts at word 2 n_records sum_{q<p} W_q, record r's row is [carrier W_p |
 * reference W_p]; valid: HOST uint32, population p at n_records sum_{q<p}
 * W_q, record r's row W_p words (allele >= 0).  site_flags (nullable): HOST
 * uint8 [n_records] over every haplotype of the VCF: bit 0 an allele 0, bit
 * 1 an allele 1, bit 2 an allele >= 2, bit 3 a missing allele.  pop_flags
 * (nullable): HOST uint8 [n_records][n_pops]: bit 0 a missing allele, bit 1
 * an allele outside {0, 1} in the population's rows.  pos: int64 POS. */
int pgld_vcf_pack_gt(const char* text, int64_t len, int32_t n_samples, int64_t n_records,
                     const int32_t* hap_rows, const int32_t* pop_offsets, int32_t n_pops,
                     uint32_t* planes, uint32_t* valid, uint8_t* site_flags, uint8_t* pop_flags,
                     int64_t* pos);

/* ----------------------------------------------------------------------
 * Measurement (no counterpart in the reference, which publishes no kernel
 * timings).
 * ---------------------------------------------------------------------- */
/* Tensor-core configuration of h (the autotuner's knobs): tile layout -- 0
 * automatic, 1 tiles of 64 x 64 SNPs (M = N = 128 MMAs; binned: one
 * accumulator per population), 2 tiles of 64 x 128 SNPs (M = 128, N = 256
 * MMAs; binned: both populations' counts in one accumulator, populations of
 * at most 2,016 haplotypes).  Automatic: layout 2 for the binned
 * two-population sums and the window sums, layout 1 for the per-pair
 * outputs.  And a cap on the pipeline stages of the tensor-core kernels
 * (0: as many as shared memory holds).  No counterpart in the
 * reference, whose chunk sizes come from free device memory
 * (ld_pipeline.py:16-49, _memutil.py:6-52). */
int pgld_set_tc_config(pgld_handle h, int32_t layout, int32_t max_stages);

/* Turn per-launch timing of each call's dominant kernel (the band, window
 * or tensor-core kernel) on or off for h; turning it on clears the list. */
int pgld_set_kernel_timing(pgld_handle h, int32_t on);
/* Device times (ms, CUDA events on the call's stream) of the dominant-kernel
 * launches timed since the last read, oldest first: up to capacity written
 * to ms_out, the number timed in *n_out; clears the list (synchronises). */
int pgld_kernel_times(pgld_handle h, float* ms_out, int32_t capacity, int32_t* n_out);
/* Throughput of the tensor-core instruction of the tcgen05 kernels: every
 * SM issues mmas_per_sm E4M3 tcgen05.mma (M = 128, N = n_cols in {64, 128,
 * 256}, K = 32, float32 accumulators) from operands resident in shared
 * memory, `launches` times back to back.  *ms_out = elapsed device time,
 * *flops_out = 2 * 128 * n_cols * 32 * mmas_per_sm * SMs * launches
 * (synchronises). */
int pgld_tc_mma_rate(pgld_handle h, int32_t n_cols, int64_t mmas_per_sm, int32_t launches,
                     float* ms_out, double* flops_out, void* stream);

/* pgld_hap_binned_sums for callers that cannot allocate device memory.
 * No counterpart in the reference.  Some callers of this library cannot call
 * cudaMalloc: a host application that hands every byte of the device to its
 * own pool allocator (a cudaMalloc outside the pool fails once the pool has
 * reserved the device, or is forbidden by the host), or a latency-bound loop
 * that cannot afford cudaMalloc's implicit device-wide synchronisation.  This
 * entry point needs no handle and allocates nothing: the tile work list and
 * its prefix-sum partials live in a 4 MiB file-scope static device array that
 * every GPU loading the library holds until the process exits, which limits a
 * call to 16,771,040 SNPs (larger panels are rejected with
 * PGLD_ERR_TOO_LARGE before any work is queued).  The caller still passes
 * every input and output buffer; sums and pair_counts are zeroed by the call.
 * The first call on a device resolves the static array's device address and
 * fills constant term tables, so make it before any stream capture.  All
 * calls on a device share the one array: calls that overlap on the GPU (other
 * streams or host threads) race and must be serialised by the caller.
 * Plain form only; arguments and results as pgld_hap_binned_sums. */
int pgld_hap_binned_sums_noalloc(int device, const pgld_hap_panel* panel, const double* pos,
                                 double max_dist, const double* bin_coord, const double* bins,
                                 int32_t n_bins, double* sums, int64_t* pair_counts,
                                 void* stream);
/* Device error word of the last allocation-free call on `device` (each call
 * clears it first; 0 = no error, a nonzero code means the call met a corrupt
 * work list and skipped that work), read and cleared through symbol copies,
 * without an allocation.  Waits for the device's earlier work.  No
 * counterpart in the reference. */
int pgld_noalloc_status(int device, int32_t* code_out);

#ifdef __cplusplus
}
#endif
#endif /* PGLD_H */
