// sched.cu -- learned per-level scheduler (placeholder until the model lands).
#include "engine.h"

namespace bfsgb {

bfs_status run_learned(bfs_graph *, const bfs_options &, LevelTimer *, uint32_t *) {
  return fail(BFS_ERR_UNSUPPORTED, "learned scheduler not available");
}
void free_sched(bfs_graph *) {}

}  // namespace bfsgb
