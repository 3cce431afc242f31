// Host build of the float32 statistic epilogue (pg_gpu_gb300/csrc/pgld_epilogue.cuh)
// for tests/test_epilogue_cpu.py: the same formulas and reciprocal tables as the
// device kernels, with the host's correctly rounded conversions in place of the
// device bit tricks.
#include <vector>

#include "../../pg_gpu_gb300/csrc/pgld_epilogue2.cuh"

extern "C" void pgld_check_stats(const int* counts, const int* n, int N, int P, float* out) {
  using namespace pgld::fast;
  int nmax = 0;
  for (int k = 0; k < N * 2; ++k) nmax = n[k] > nmax ? n[k] : nmax;
  std::vector<float> tab(4 * (nmax + 1));
  for (int v = 0; v <= nmax; ++v)
    recip_entry(v, &tab[v], &tab[(nmax + 1) + v], &tab[2 * (nmax + 1) + v], &tab[3 * (nmax + 1) + v]);
  Recip T{&tab[0], &tab[nmax + 1], &tab[2 * (nmax + 1)], &tab[3 * (nmax + 1)]};
  for (int k = 0; k < N; ++k) {
    const int* c = counts + 8 * k;
    Pop p = make((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
    if (P == 1) {
      stats1(p, T, out + 3 * k);
    } else {
      Pop q = make((float)c[4], (float)c[5], (float)c[6], (float)c[7]);
      stats2(p, q, T, out + 15 * k);
    }
  }
}

// the packed two-pair form: rows k and N-1-k share one float2 evaluation; the
// reciprocals come from the interleaved float4 table of the tensor-core kernel
extern "C" void pgld_check_stats2(const int* counts, const int* n, int N, int P, float* out) {
  using namespace pgld::fast;
  namespace f2 = pgld::fast2;
  int nmax = 0;
  for (int k = 0; k < N * 2; ++k) nmax = n[k] > nmax ? n[k] : nmax;
  std::vector<float4> tab(nmax + 1);
  for (int v = 0; v <= nmax; ++v) f2::recip_entry4(v, &tab[v]);
  const float4* T = tab.data();
  const int S = P == 1 ? 3 : 15;
  for (int k = 0; k < N; ++k) {
    const int* a = counts + 8 * k;
    const int* b = counts + 8 * (N - 1 - k);
    auto v = [&](int m) { return make_float2((float)a[m], (float)b[m]); };
    f2::Pop p = f2::make(v(0), v(1), v(2), v(3));
    float2 o[15];
    if (P == 1) {
      f2::stats1(p, T, o);
    } else {
      f2::Pop q = f2::make(v(4), v(5), v(6), v(7));
      f2::stats2(p, q, T, o);
    }
    for (int s = 0; s < S; ++s) out[S * k + s] = o[s].x;
  }
}
