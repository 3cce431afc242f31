// Host build of the float32 statistic epilogue (pg_gpu_gb300/csrc/pgld_epilogue.cuh)
// for tests/test_epilogue_cpu.py: the same formulas as the device kernels, with
// the host's correctly rounded conversions in place of the device bit tricks.
#include "../../pg_gpu_gb300/csrc/pgld_epilogue.cuh"

extern "C" void pgld_check_stats(const int* counts, const int* n, int N, int P, float* out) {
  using namespace pgld::fast;
  for (int k = 0; k < N; ++k) {
    const int* c = counts + 8 * k;
    Pop p = make(c[0], c[1], c[2], c[3], n[2 * k]);
    if (P == 1) {
      stats1(p, out + 3 * k);
    } else {
      Pop q = make(c[4], c[5], c[6], c[7], n[2 * k + 1]);
      stats2(p, q, out + 15 * k);
    }
  }
}
