// rt_split.h -- split-precision (BF16 slices on the tensor cores) variants
// of the four GEMMs of the transformation.
#pragma once
#include <string>

#include "rt_internal.h"
#include "rt_kernels.h"

namespace rt {

// K per split of the adjoint's long contraction (one exponent per block)
constexpr int SPLIT_LONG_BLOCK = 768;
void split_prepare_constants(rt_ctx* c);
// Message for a GEMM status word; *unconfirmed is set when the aborted
// launch could not confirm that its MMAs and copies had finished.
std::string split_status_text(int e, bool* unconfirmed);
double split_stageA_bytes_per_pair(rt_ctx* c);
double split_stageB_bytes_per_item(rt_ctx* c);
void split_alloc_work(rt_ctx* c, int pair_chunk, int item_chunk);
// bytes the work arena of split_alloc_work holds now (0 before the first)
size_t split_work_bytes(rt_ctx* c);
// GEMM1 operand buffers the bucket expansion fills (slices, row exponents)
__nv_bfloat16* split_a1_slices(rt_ctx* c);
int* split_a1_exps(rt_ctx* c);
void split_gemm1(rt_ctx* c, const G1Group& g, int npc, const EpiHA& epi, int* launches);
void split_gemm24(rt_ctx* c, const double* B, int K, long long N, const EpiRowMajor& epi,
                  int* launches);
void split_gemm3(rt_ctx* c, int comp, const double* m3, int nc, int nij, const EpiRK& epi,
                 int* launches);
// GEMM2 over the RI blocks the Kramers selection reads (3/4 of the full product)
void split_gemm2_kramers(rt_ctx* c, const double* B, int K, long long N, const EpiRowMajor& epi,
                         int* launches);
void split_release(rt_ctx* c);
// Gaunt (Breit) transformation
void split_gemm2_breit(rt_ctx* c, const double* B, int K, long long N, const EpiRowMajor& ria,
                       const EpiRowMajor& ri2, int* launches);
void split_gemm3_op(rt_ctx* c, int op, int kcomp, const double* m3, int nrow, int ncol, int nij,
                    const EpiRK& e, int* launches);
void split_gemm4_op(rt_ctx* c, int op, const double* B, int K, long long N, const EpiRowMajor& e,
                    int* launches);
// operand slicing of GEMM2/4 and GEMM3 on stream st (the GEMM itself apart)
void split_prep_gemm24(rt_ctx* c, const double* Bsrc, int K, long long N, cudaStream_t st,
                       int* launches);
void split_prep_gemm3(rt_ctx* c, const double* m3, int nc, int nij, cudaStream_t st,
                      int* launches);
// grouped launches of one GEMM stage over many transforms (kind 0: GEMM1,
// 1: GEMM2/4, 2: GEMM3); tables are built once and launched many times
struct SplitGroup;
SplitGroup* split_group_new(int kind);
void split_group_add_gemm1(SplitGroup* g, rt_ctx* c, const G1Group& gg, int npc, const EpiHA& e);
void split_group_add_gemm24(SplitGroup* g, rt_ctx* c, int K, long long N, const EpiRowMajor& e);
void split_group_add_gemm3(SplitGroup* g, rt_ctx* c, int comp, int nc, int nij, const EpiRK& e);
void split_group_add_gemm2_kramers(SplitGroup* g, rt_ctx* c, int K, long long N, const EpiRowMajor& e);
void split_group_build(SplitGroup* g, rt_ctx* c0);
void split_group_launch(SplitGroup* g, int bn, cudaStream_t st, int* err);
int split_group_size(const SplitGroup* g);
// shape class of a group for the tile-width cache: kind, slices, problems,
// tiles at both widths, executed FLOPs rounded to a power of two
std::string split_group_shape(const SplitGroup* g);
double split_group_flops(const SplitGroup* g, bool executed);
void split_group_free(SplitGroup* g);
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
