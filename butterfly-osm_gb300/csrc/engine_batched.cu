// engine_batched.cu — batched engine (shared-memory subtrees). Filled in below.
#include "engine.cuh"

namespace bf {

bf_status batched_prepare(Graph* g, uint32_t S_max) {
  (void)g;
  (void)S_max;
  return BF_OK;
}

bf_status batched_matrix(Graph* g, const uint32_t* d_src, uint64_t S, const uint32_t* d_tgt,
                         uint64_t T, uint32_t threshold, uint32_t* d_out, cudaStream_t st,
                         bf_stats* stats) {
  (void)g; (void)d_src; (void)S; (void)d_tgt; (void)T; (void)threshold; (void)d_out; (void)st;
  (void)stats;
  set_error("batched engine not ready");
  return BF_ERR_UNSUPPORTED;
}

}  // namespace bf
