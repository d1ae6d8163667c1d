// bh.cu -- Barnes-Hut on the GPU (placeholder until the tree pipeline lands).
#include "gvs_internal.cuh"

namespace gvs {
gvs_status bh_forces(Ctx *c, double, double, int, bool) {
    return fail(c, GVS_ERR_STATE, "Barnes-Hut path not available in this build");
}
gvs_status tree_build(Ctx *c) { return fail(c, GVS_ERR_STATE, "tree build not available in this build"); }
void tree_free(Ctx *) {}
}  // namespace gvs
