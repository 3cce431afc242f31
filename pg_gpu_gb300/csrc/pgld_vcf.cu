// Native VCF GT reader (host code): phased or unphased genotypes of a VCF text
// into the int8 haplotype matrix of HaplotypeMatrix.from_vcf (rows: every
// sample's first allele, then every sample's second allele;
// haplotype_matrix.py:293-404) and the positions, without a Python loop per
// genotype.  Alleles: '.' (or an empty field) is -1, a number its value
// (clipped to 127), a haploid call has -1 as its second allele.
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

// one data record: POS and the GT alleles of the selected samples
// (col[s] = output column of VCF sample s, -1 = not selected); false if the
// record has fewer than 9 + n_samples fields
static bool parse_record(const char* p, const char* lend, int32_t n_samples, const int32_t* col,
                         int32_t n_sel, int64_t n_records, int64_t r, int8_t* hap,
                         int64_t* pos) {
  // CHROM, then POS
  while (p < lend && *p != '\t') ++p;
  if (p == lend) return false;
  ++p;
  int64_t v = 0;
  for (; p < lend && *p >= '0' && *p <= '9'; ++p) v = v * 10 + (*p - '0');
  pos[r] = v;
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
    const int32_t c = col[s];
    if (c < 0) continue;
    // GT: allele, then '/' or '|' and a second allele, ending at ':' / tab
    const char* a0 = p;
    while (p < lend && *p != '/' && *p != '|' && *p != ':' && *p != '\t') ++p;
    hap[(int64_t)c * n_records + r] = allele(a0, p);
    int8_t second = -1;
    if (p < lend && (*p == '/' || *p == '|')) {
      const char* a1 = ++p;
      while (p < lend && *p != '/' && *p != '|' && *p != ':' && *p != '\t') ++p;
      second = allele(a1, p);
    }
    hap[(int64_t)(n_sel + c) * n_records + r] = second;
  }
  return true;
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
  // record lines: [start, end without '\r')
  std::vector<const char*> rb, re;
  rb.reserve((size_t)n_records);
  re.reserve((size_t)n_records);
  for (const char *p = text, *end = text + len; p < end;) {
    const char* le = line_end(p, end);
    const char* lend = (le > p && le[-1] == '\r') ? le - 1 : le;
    if (lend > p && *p != '#') {
      if ((int64_t)rb.size() >= n_records) return PGLD_ERR_INVALID_ARG;
      rb.push_back(p);
      re.push_back(lend);
    }
    p = le + 1;
  }
  if ((int64_t)rb.size() != n_records) return PGLD_ERR_INVALID_ARG;
  // records in parallel: each writes only its own column of hap
  const int64_t bytes = len;
  int nt = (int)std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()),
                                   std::max<int64_t>(1, bytes >> 22));
  nt = (int)std::min<int64_t>(nt, std::max<int64_t>(n_records, 1));
  std::atomic<int> bad{0};
  auto work = [&](int t) {
    const int64_t r0 = n_records * t / nt, r1 = n_records * (t + 1) / nt;
    for (int64_t r = r0; r < r1; ++r)
      if (!parse_record(rb[r], re[r], n_samples, col.data(), n_sel, n_records, r, hap, pos)) {
        bad.store(1);
        return;
      }
  };
  std::vector<std::thread> th;
  th.reserve((size_t)nt);
  for (int t = 1; t < nt; ++t) {
    try {
      th.emplace_back(work, t);
    } catch (...) {
      break;  // the chunks without a thread run below
    }
  }
  for (int t = 1 + (int)th.size(); t < nt; ++t) work(t);
  work(0);
  for (auto& x : th) x.join();
  return bad.load() ? PGLD_ERR_INVALID_ARG : PGLD_OK;
}
