// Native VCF GT reader (host code): phased or unphased genotypes of a VCF text
// into the int8 haplotype matrix of HaplotypeMatrix.from_vcf (rows: every
// sample's first allele, then every sample's second allele;
// haplotype_matrix.py:293-404) and the positions, without a Python loop per
// genotype (pgld_vcf_parse_gt), or straight into the populations' carrier /
// reference / validity bit planes with per-site and per-population flags,
// skipping the int8 matrix (pgld_vcf_pack_gt).  Alleles: '.' (or an empty
// field) is -1, a number its value (clipped to 127), a haploid call has -1 as
// its second allele.  Records are parsed on all host threads, each thread a
// contiguous range of records writing only their own rows.
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/pgld.h"

namespace {

inline const char* line_end(const char* p, const char* end) {
  const void* q = memchr(p, '\n', (size_t)(end - p));
  return q ? (const char*)q : end;
}

inline int8_t allele(const char* b, const char* e) {
  if (b == e || *b == '.') return -1;
  int v = 0;
  for (const char* q = b; q < e && *q >= '0' && *q <= '9'; ++q) {
    v = v * 10 + (*q - '0');
    if (v > 127) return 127;
  }
  return (int8_t)v;
}

}  // namespace

extern "C" int pgld_vcf_scan(const char* text, int64_t len, int32_t* n_samples,
                             int64_t* n_records) {
  if (!text || len < 0 || !n_samples || !n_records) return PGLD_ERR_INVALID_ARG;
  const char* p = text;
  const char* end = text + len;
  int32_t ns = -1;
  int64_t nr = 0;
  while (p < end) {
    const char* le = line_end(p, end);
    if (le > p && *p == '#') {
      if (le - p >= 6 && memcmp(p, "#CHROM", 6) == 0) {
        int tabs = 0;
        for (const char* q = p; q < le; ++q) tabs += (*q == '\t');
        ns = tabs >= 9 ? tabs - 8 : 0;
      }
    } else if (le > p && !(le - p == 1 && *p == '\r')) {
      ++nr;
    }
    p = le + 1;
  }
  if (ns < 0) return PGLD_ERR_INVALID_ARG;  // no #CHROM header line
  *n_samples = ns;
  *n_records = nr;
  return PGLD_OK;
}

// one data record: POS, then on_gt(s, allele 0, allele 1) for every VCF
// sample s in column order; false if the record has fewer than 9 + n_samples
// fields
template <class OnGt>
static bool for_each_gt(const char* p, const char* lend, int32_t n_samples, int64_t* pos_out,
                        OnGt&& on_gt) {
  // CHROM, then POS
  while (p < lend && *p != '\t') ++p;
  if (p == lend) return false;
  ++p;
  int64_t v = 0;
  for (; p < lend && *p >= '0' && *p <= '9'; ++p) v = v * 10 + (*p - '0');
  *pos_out = v;
  // skip to the first sample field (after the 9th tab)
  for (int t = 1; t < 9; ++t) {
    while (p < lend && *p != '\t') ++p;
    if (p == lend) return n_samples == 0;
    ++p;
  }
  for (int32_t s = 0; s < n_samples; ++s) {
    if (s > 0) {
      while (p < lend && *p != '\t') ++p;  // rest of the previous field
      if (p == lend) return false;
      ++p;
    }
    // GT: allele, then '/' or '|' and a second allele, ending at ':' / tab
    const char* a0 = p;
    while (p < lend && *p != '/' && *p != '|' && *p != ':' && *p != '\t') ++p;
    const int8_t first = allele(a0, p);
    int8_t second = -1;
    if (p < lend && (*p == '/' || *p == '|')) {
      const char* a1 = ++p;
      while (p < lend && *p != '/' && *p != '|' && *p != ':' && *p != '\t') ++p;
      second = allele(a1, p);
    }
    on_gt(s, first, second);
  }
  return true;
}

// the record lines of a VCF text ([start, end without '\r')); false unless
// there are exactly n_records
static bool record_lines(const char* text, int64_t len, int64_t n_records,
                         std::vector<const char*>& rb, std::vector<const char*>& re) {
  rb.reserve((size_t)n_records);
  re.reserve((size_t)n_records);
  for (const char *p = text, *end = text + len; p < end;) {
    const char* le = line_end(p, end);
    const char* lend = (le > p && le[-1] == '\r') ? le - 1 : le;
    if (lend > p && *p != '#') {
      if ((int64_t)rb.size() >= n_records) return false;
      rb.push_back(p);
      re.push_back(lend);
    }
    p = le + 1;
  }
  return (int64_t)rb.size() == n_records;
}

// work(r0, r1) over contiguous record ranges on the host threads (at most one
// per 4 MB of text); false if any range failed
template <class Work>
static bool parallel_records(int64_t len, int64_t n_records, Work&& work) {
  int nt = (int)std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()),
                                   std::max<int64_t>(1, len >> 22));
  nt = (int)std::min<int64_t>(nt, std::max<int64_t>(n_records, 1));
  std::atomic<int> bad{0};
  auto run = [&](int t) {
    const int64_t r0 = n_records * t / nt, r1 = n_records * (t + 1) / nt;
    if (!work(r0, r1)) bad.store(1);
  };
  std::vector<std::thread> th;
  th.reserve((size_t)nt);
  for (int t = 1; t < nt; ++t) {
    try {
      th.emplace_back(run, t);
    } catch (...) {
      break;  // the ranges without a thread run below
    }
  }
  for (int t = 1 + (int)th.size(); t < nt; ++t) run(t);
  run(0);
  for (auto& x : th) x.join();
  return bad.load() == 0;
}

extern "C" int pgld_vcf_parse_gt(const char* text, int64_t len, int32_t n_samples,
                                 int64_t n_records, const int32_t* sample_cols, int32_t n_sel,
                                 int8_t* hap, int64_t* pos) {
  if (!text || len < 0 || n_samples < 0 || n_records < 0 || n_sel < 0 || !hap || !pos)
    return PGLD_ERR_INVALID_ARG;
  // output column of every VCF sample (-1: not selected)
  std::vector<int32_t> col((size_t)n_samples, sample_cols ? -1 : 0);
  if (sample_cols) {
    for (int32_t k = 0; k < n_sel; ++k) {
      if (sample_cols[k] < 0 || sample_cols[k] >= n_samples) return PGLD_ERR_INVALID_ARG;
      col[sample_cols[k]] = k;
    }
  } else {
    if (n_sel != n_samples) return PGLD_ERR_INVALID_ARG;
    for (int32_t s = 0; s < n_samples; ++s) col[s] = s;
  }
  std::vector<const char*> rb, re;
  if (!record_lines(text, len, n_records, rb, re)) return PGLD_ERR_INVALID_ARG;
  // records in parallel: each writes only its own column of hap
  const bool ok = parallel_records(len, n_records, [&](int64_t r0, int64_t r1) {
    for (int64_t r = r0; r < r1; ++r) {
      const bool rec_ok = for_each_gt(rb[r], re[r], n_samples, pos + r,
                                      [&](int32_t smp, int8_t a0, int8_t a1) {
                                        const int32_t c = col[smp];
                                        if (c < 0) return;
                                        hap[(int64_t)c * n_records + r] = a0;
                                        hap[(int64_t)(n_sel + c) * n_records + r] = a1;
                                      });
      if (!rec_ok) return false;
    }
    return true;
  });
  return ok ? PGLD_OK : PGLD_ERR_INVALID_ARG;
}

extern "C" int pgld_vcf_pack_gt(const char* text, int64_t len, int32_t n_samples,
                                int64_t n_records, const int32_t* hap_rows,
                                const int32_t* pop_offsets, int32_t n_pops, uint32_t* planes,
                                uint32_t* valid, uint8_t* site_flags, uint8_t* pop_flags,
                                int64_t* pos) {
  if (!text || len < 0 || n_samples < 0 || n_records < 0 || n_pops < 0 || !pos ||
      (n_pops > 0 && (!hap_rows || !pop_offsets || !planes || !valid)))
    return PGLD_ERR_INVALID_ARG;
  const int64_t n_hap = 2 * (int64_t)n_samples;
  // every VCF haplotype's destinations (population, bit), as CSR lists
  std::vector<int64_t> wbase((size_t)n_pops + 1, 0);  // words of the populations before p
  std::vector<int32_t> W((size_t)n_pops);
  for (int32_t p = 0; p < n_pops; ++p) {
    const int32_t n_rows = pop_offsets[p + 1] - pop_offsets[p];
    if (pop_offsets[p] < 0 || n_rows < 0) return PGLD_ERR_INVALID_ARG;
    W[p] = std::max(1, (n_rows + 31) / 32);
    wbase[p + 1] = wbase[p] + W[p];
  }
  std::vector<int32_t> first((size_t)n_hap + 1, 0);
  for (int32_t p = 0; p < n_pops; ++p)
    for (int32_t k = pop_offsets[p]; k < pop_offsets[p + 1]; ++k) {
      const int32_t h = hap_rows[k];
      if (h < 0 || h >= n_hap) return PGLD_ERR_INVALID_ARG;
      ++first[(size_t)h + 1];
    }
  for (int64_t h = 0; h < n_hap; ++h) first[h + 1] += first[h];
  std::vector<int32_t> dpop((size_t)first[n_hap]), dbit((size_t)first[n_hap]);
  {
    std::vector<int32_t> fill(first.begin(), first.end() - 1);
    for (int32_t p = 0; p < n_pops; ++p)
      for (int32_t k = pop_offsets[p]; k < pop_offsets[p + 1]; ++k) {
        const int32_t at = fill[hap_rows[k]]++;
        dpop[at] = p;
        dbit[at] = k - pop_offsets[p];
      }
  }
  std::vector<const char*> rb, re;
  if (!record_lines(text, len, n_records, rb, re)) return PGLD_ERR_INVALID_ARG;
  const bool ok = parallel_records(len, n_records, [&](int64_t r0, int64_t r1) {
    std::vector<uint8_t> pf((size_t)std::max(n_pops, 1));
    for (int64_t r = r0; r < r1; ++r) {
      for (int32_t p = 0; p < n_pops; ++p) {
        std::memset(planes + 2 * (n_records * wbase[p] + r * W[p]), 0, 8 * (size_t)W[p]);
        std::memset(valid + n_records * wbase[p] + r * W[p], 0, 4 * (size_t)W[p]);
        pf[p] = 0;
      }
      uint8_t sf = 0;
      auto put = [&](int64_t h, int8_t v) {
        sf |= v == 0 ? 1 : v == 1 ? 2 : v > 1 ? 4 : 8;
        for (int32_t d = first[h]; d < first[h + 1]; ++d) {
          const int32_t p = dpop[d], k = dbit[d];
          const uint32_t bit = 1u << (k & 31);
          uint32_t* row = planes + 2 * (n_records * wbase[p] + r * W[p]);
          if (v == 1) row[k >> 5] |= bit;
          if (v == 0) row[W[p] + (k >> 5)] |= bit;
          if (v >= 0) valid[n_records * wbase[p] + r * W[p] + (k >> 5)] |= bit;
          pf[p] |= v < 0 ? 1 : v > 1 ? 2 : 0;
        }
      };
      const bool rec_ok = for_each_gt(rb[r], re[r], n_samples, pos + r,
                                      [&](int32_t smp, int8_t a0, int8_t a1) {
                                        put(smp, a0);
                                        put((int64_t)n_samples + smp, a1);
                                      });
      if (!rec_ok) return false;
      if (site_flags) site_flags[r] = sf;
      if (pop_flags)
        for (int32_t p = 0; p < n_pops; ++p) pop_flags[r * n_pops + p] = pf[p];
    }
    return true;
  });
  return ok ? PGLD_OK : PGLD_ERR_INVALID_ARG;
}
