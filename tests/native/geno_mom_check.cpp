// Host build of the centred-moment genotype estimators
// (pg_gpu_gb300/csrc/pgld_geno_mom.cuh) for tests/test_geno_mom_cpu.py: per
// count row the nine moments, the counts recovered from them, and the exact
// int64 numerators of DD, Dz, pi2 and the Rogers-Huff cov^2 / var_I var_J.
#include "../../pg_gpu_gb300/csrc/pgld_geno_mom.cuh"

extern "C" void pgld_check_geno_mom(const int* counts, int N, int* mom, int* back,
                                    long long* num) {
  using namespace pgld::gmom;
  for (int k = 0; k < N; ++k) {
    const Mom o = from_counts(counts + 9 * k);
    for (int x = 0; x < 9; ++x) mom[9 * k + x] = o.m[x];
    to_counts(o, back + 9 * k);
    const Terms t = terms(o);
    const RHm r = rh(o);
    long long* q = num + 6 * k;
    q[0] = dd_num(o, t);
    q[1] = dz_num(o, t);
    q[2] = pi2_num(o, t);
    q[3] = d4(o.m[0]);
    q[4] = r.cov2;
    q[5] = r.den;
  }
}
