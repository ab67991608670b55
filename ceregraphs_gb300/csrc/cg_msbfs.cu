// Multi-source BFS (placeholder until the lane kernels land).
#include "cg_internal.cuh"
namespace cg {
int msbfs_prepare(cg_graph *g, int lane_words, int64_t out_elems) {
  (void)g; (void)lane_words; (void)out_elems;
  return CG_ERR_NOT_SUPPORTED;
}
void msbfs_release(cg_graph *g) { (void)g; }
int msbfs_launch(cg_graph *g, const int64_t *roots, int32_t k, int32_t *d_levels,
                 int32_t *d_parents) {
  (void)g; (void)roots; (void)k; (void)d_levels; (void)d_parents;
  return CG_ERR_NOT_SUPPORTED;
}
}  // namespace cg
