// Ozaki-split contraction: placeholder until the tcgen05 kernel lands.
#include "ozaki.cuh"

namespace hsdla {

static const char *g_oz_err = "";

int ozaki_plan_init(OzakiPlan &oz, int num_slices, double target) {
    oz.num_slices = num_slices;
    oz.target = target;
    return HSDLA_OK;
}
int64_t ozaki_workspace_bytes(const OzakiPlan &, int64_t, int64_t) { return 0; }
int ozaki_contract(OzakiPlan &, const double2 *, const double2 *, const double *, int64_t, int64_t, double2 *,
                   double2 *, int64_t, void *, cudaStream_t, int *) {
    g_oz_err = "Ozaki path not built";
    return HSDLA_ERR_UNSUPPORTED;
}
int ozaki_herkx(OzakiPlan &, const double2 *, int64_t, const double2 *, int64_t, const double *, int64_t, int64_t,
                double2 *, int64_t, void *, cudaStream_t, int *) {
    g_oz_err = "Ozaki path not built";
    return HSDLA_ERR_UNSUPPORTED;
}
int ozaki_check_device_error(OzakiPlan &) { return HSDLA_OK; }
const char *ozaki_last_error() { return g_oz_err; }

}  // namespace hsdla
