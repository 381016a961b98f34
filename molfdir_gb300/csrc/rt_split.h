// rt_split.h -- split-precision (BF16 slices on the tensor cores) variants
// of the four GEMMs of the transformation.
#pragma once

#include "rt_internal.h"
#include "rt_kernels.h"

namespace rt {

void split_prepare_constants(rt_ctx* c);
double split_stageA_bytes_per_pair(rt_ctx* c);
double split_stageB_bytes_per_item(rt_ctx* c);
void split_alloc_work(rt_ctx* c, int pair_chunk, int item_chunk);
// GEMM1 operand buffers the bucket expansion fills (slices, row exponents)
__nv_bfloat16* split_a1_slices(rt_ctx* c);
int* split_a1_exps(rt_ctx* c);
void split_gemm1(rt_ctx* c, const G1Group& g, int npc, const EpiHA& epi, int* launches);
void split_gemm24(rt_ctx* c, const double* B, int K, long long N, const EpiRowMajor& epi,
                  int* launches);
void split_gemm3(rt_ctx* c, int comp, const double* m3, int nc, int nij, const EpiRK& epi,
                 int* launches);
void split_release(rt_ctx* c);
// adjoint: X GEMM of one component and the split-K contraction
void split_adj_x(rt_ctx* c, int comp, const double* m3, int nc, int nij, double* x,
                 __nv_bfloat16* sl, int* ex, int* launches);
long long split_adj_kpad(long long K);
int split_adj_contract(rt_ctx* c, const double* x, int rows, long long Kx, const double* ghat_t,
                       __nv_bfloat16* a_sl, int* a_ex, __nv_bfloat16* b_sl, int* b_ex, double* part,
                       int* launches);
// executed FLOPs per algorithmic FLOP of a split GEMM (slice products)
double split_flop_factor(rt_ctx* c);
// raise if a split GEMM gave up waiting (bounded-wait timeout)
void split_check(rt_ctx* c);

}  // namespace rt
