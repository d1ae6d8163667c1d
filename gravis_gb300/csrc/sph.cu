// sph.cu -- SPH on the GPU (placeholder until the SPH pipeline lands).
#include "gvs_internal.cuh"

namespace gvs {
gvs_status sph_compute(Ctx *c, const gvs_sph_params *) {
    return fail(c, GVS_ERR_STATE, "SPH path not available in this build");
}
gvs_status sph_timestep(Ctx *c, const gvs_sph_params *, double *) {
    return fail(c, GVS_ERR_STATE, "SPH path not available in this build");
}
void sph_free(Ctx *) {}
}  // namespace gvs
