// Ozaki-split FP64 contraction on the FP8 (e4m3) tensor cores of sm_103a.
#pragma once

#include "common.cuh"

namespace hsdla {

constexpr int kOzMaxSlices = 12;

struct OzakiPlan {
    int num_slices = 0;          // digit slices per operand
    double target = 1e-13;
    int *d_error = nullptr;      // device error word (bounded waits)
};

int ozaki_plan_init(OzakiPlan &oz, int num_slices, double target);
int64_t ozaki_workspace_bytes(const OzakiPlan &oz, int64_t K, int64_t n);
// S = (diag(wsqrt) C)^H (diag(wsqrt) C), H = C^H X; lower triangles; C, X: K x G, ld K.
int ozaki_contract(OzakiPlan &oz, const double2 *C, const double2 *X, const double *wsqrt, int64_t K, int64_t G,
                   double2 *S, double2 *H, int64_t ldo, void *ws, cudaStream_t st, int *launches);
// OUT = P^H diag(w) Q, lower triangle (standalone component).
int ozaki_herkx(OzakiPlan &oz, const double2 *P, int64_t ldp, const double2 *Q, int64_t ldq, const double *w,
                int64_t K, int64_t n, double2 *out, int64_t ldo, void *ws, cudaStream_t st, int *launches);
int ozaki_check_device_error(OzakiPlan &oz);
const char *ozaki_last_error();

}  // namespace hsdla
