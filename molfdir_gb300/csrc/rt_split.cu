// rt_split.cu -- split-precision GEMMs (under construction).
#include "rt_split.h"

namespace rt {

static void not_built() { throw Error(RT_ERR_USER, "split-BF16 path not available in this build"); }
void split_prepare_constants(rt_ctx*) { not_built(); }
double split_stageA_bytes_per_pair(rt_ctx*) { return 0.0; }
double split_stageB_bytes_per_item(rt_ctx*) { return 0.0; }
void split_alloc_work(rt_ctx*, int, int) { not_built(); }
void split_prepare_g3(rt_ctx*, int*) { not_built(); }
void split_gemm1(rt_ctx*, const G1Group&, int, int, const EpiHA&, int*) { not_built(); }
void split_gemm24(rt_ctx*, const double*, int, long long, const EpiRowMajor&, int*) { not_built(); }
void split_gemm3(rt_ctx*, int, const double*, int, int, const EpiRK&, int*) { not_built(); }
void split_release(rt_ctx*) {}
double split_flop_factor(rt_ctx*) { return 1.0; }

}  // namespace rt
