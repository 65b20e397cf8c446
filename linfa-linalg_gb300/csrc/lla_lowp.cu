// lla_lowp.cu -- low-precision Cholesky of the equilibrated FP32 matrix for
// the mixed-precision solve: dispatch on the trailing-update form.
#include "lla_api_internal.h"
#include "lla_common.cuh"
#include "lla_kernels.h"
#include "lla_mixed.h"
#include "lla_prof.h"

namespace lla {

int lowp_factor_launch(float *L, int64_t n, int64_t ld, const lla_refine_opts &opts, int64_t *info,
                       float *diag0, double *min_ratio, Ctx *c, cudaStream_t st) {
    (void)opts;
    (void)c;
    return potrf_fast_launch<float>(L, n, ld, info, diag0, min_ratio, st);
}

}  // namespace lla
