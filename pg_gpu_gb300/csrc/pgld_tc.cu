// tcgen05 tensor-core form of the binned band kernel (sm_103a).
#include <cuda_runtime.h>

#include "pgld_band.cuh"
#include "pgld_internal.cuh"

int pgld_tc_supported(pgld_context* h, const pgld_hap_panel* panel) { return 0; }

int pgld_tc_binned(pgld_context* h, const pgld_hap_panel* panel, pgld::BandArgs& a,
                   cudaStream_t st) {
  return pgld_fail(h, PGLD_ERR_UNSUPPORTED, "tensor-core form not built");
}
