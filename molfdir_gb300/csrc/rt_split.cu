// rt_split.cu -- split-precision GEMMs of the four quarter-transformations.
//
// C = A B with A (M x K) and B (K x N) given as FP64 or float-float values is
// computed from s BF16 digit slices per operand (row scales for A, column
// scales for B; see rt_ff.cuh) on the tcgen05 tensor cores:
//
//   acc0 = sum_k a_1 b_1                       exact in FP32
//   acc1 = sum_k a_1 b_2 + a_2 b_1             exact in FP32
//   acc2 = sum_k a_1 b_3 + a_2 b_2 + a_3 b_1   exact in FP32
//   acc3 = sum_k sum_{t+u>=5} a_t b_u          FP32 (relative weight 2^-21)
//
// (exact for K <= 819 with narrow slicing and K <= 1365 with wide slicing,
// rt_ff.cuh; every operand is sliced for its GEMM's depth, split-K splits
// for theirs, and deeper GEMMs are refused)
//
// (the tensor cores' FP32 accumulation of rounded sums behaves like about
// 20 significant bits, so every product diagonal whose error would show
// above 2^-40 is kept in an exactly summed accumulator)
// (digit products with t+u > s+1 are dropped).  The epilogue recombines
// acc0+acc1+acc2 without rounding into a float-float number, applies the
// power-of-two scales and writes it; the next stage re-slices float-float
// values directly.  FP64 arithmetic, which runs at about 1/70 of the FP32
// rate on GB300, is used nowhere on this path except the final conversion
// of the MDCINT elements.
//
// GEMM kernel: persistent, one CTA per SM, 128x128 output tiles, K in steps
// of 32 (64-byte swizzled TMA tiles), two shared-memory stages holding all s
// slices of A and B; warp 0 issues TMA loads, warp 1 issues tcgen05.mma into
// four TMEM accumulators (all 512 columns), warps 2-5 drain TMEM and run the
// epilogue.  Every wait is bounded (2 s); on a timeout the kernel sets an
// error flag, stops all roles, waits for its own TMA copies and frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "rt_ff.cuh"
#include "rt_split.h"
#include "rt_umma.cuh"

namespace rt {

constexpr int SBM = 128, SBN = 128, SBK = 32, NSTAGE = 2, MAX_SLICES = 6;
constexpr unsigned long long WAIT_NS = 2000000000ull;

// Status word of a GEMM launch: the first wait that ran out (low byte), and
// two bits for an abort that could not confirm its own clean-up -- MMAs
// still writing TMEM when it was freed, or TMA copies still landing in shared
// memory when the CTA left.  Those leave the device state in doubt.
enum : int {
    ERR_TIMEOUT_EMPTY = 1,
    ERR_TIMEOUT_FULL = 2,
    ERR_TIMEOUT_TMEM = 3,
    ERR_DRAIN_UNCONFIRMED = 1 << 8,
    ERR_COPIES_UNCONFIRMED = 1 << 9
};

// ---------------------------------------------------------------------------
// slicing kernels
// ---------------------------------------------------------------------------

// Source rows of the A operand.
struct RowsF64Batched {  // GEMM1: row = r*npc + pql -> G3 row (r, c0+pql)
    const double* g3;    // group base
    long long pg_size, c0;
    int npc, nk;
    __device__ const double* row(long long i) const {
        long long r = i / npc, q = i - r * npc;
        return g3 + (r * pg_size + c0 + q) * nk;
    }
};

struct RowsFF {  // contiguous float-float rows of length K (stride ld)
    const float2* base;
    long long ld;
    __device__ const float2* row(long long i) const { return base + i * ld; }
};

// Element access of the slicing kernels: float-float value and the
// exponent S with |value| < 2^S.
__device__ __forceinline__ float2 ff_load(const double* p) { return ff_from_double(*p); }
__device__ __forceinline__ float2 ff_load(const float2* p) { return *p; }
__device__ __forceinline__ int exp_load(const double* p, int wide) { return scale_exp_f64(*p, wide); }
__device__ __forceinline__ int exp_load(const float2* p, int wide) { return scale_exp_f32(p->x, wide); }

__device__ __forceinline__ uint32_t pack_bf16x2(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// A operand: one warp per row, four consecutive k per lane; output
// [s][M][Kp] BF16 (K-major) plus the row exponents.
template <int NS, class Src>
__global__ void __launch_bounds__(256) k_slice_rows(Src src, long long M, int K, int Kp,
                                                    __nv_bfloat16* __restrict__ out,
                                                    int* __restrict__ exps) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long i = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < M;
         i += warps) {
        const auto* p = src.row(i);
        const int wide = slicing_wide(K);
        int S = -2000;
        for (int k = lane; k < K; k += 32) S = max(S, exp_load(p + k, wide));
        for (int o = 16; o; o >>= 1) S = max(S, __shfl_xor_sync(0xffffffffu, S, o));
        if (lane == 0) exps[i] = S;
        const float sc = pow2f_safe(-S);
        for (int k0 = lane * 4; k0 < Kp; k0 += 128) {
            __nv_bfloat16 d[4][NS];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float2 v = make_float2(0.f, 0.f);
                if (k0 + j < K && S > -1000) v = ff_load(p + k0 + j);
                ff_digits<NS>(v.x * sc, v.y * sc, d[j]);
            }
#pragma unroll
            for (int t = 0; t < NS; ++t) {
                uint2 w = make_uint2(pack_bf16x2(d[0][t], d[1][t]), pack_bf16x2(d[2][t], d[3][t]));
                *reinterpret_cast<uint2*>(out + ((long long)t * M + i) * Kp + k0) = w;
            }
        }
    }
}

// B operand: a block handles 32 columns of a K x N float-float matrix:
// column exponents, then digits transposed through shared memory to
// [s][N][Kp] (K-major), 64 k per tile.
template <int NS>
__global__ void __launch_bounds__(256) k_slice_cols(const float2* __restrict__ src, long long ld,
                                                    int K, long long N, int Kp,
                                                    int* __restrict__ exps,
                                                    __nv_bfloat16* __restrict__ out) {
    __shared__ __nv_bfloat16 tile[NS][32][66];
    __shared__ int part[8][32];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const long long n0 = (long long)blockIdx.x * 32;
    const long long n = n0 + tx;
    int S = -2000;
    const int wide = slicing_wide(K);
    if (n < N)
        for (int k = ty; k < K; k += 8) S = max(S, scale_exp_f32(src[(long long)k * ld + n].x, wide));
    part[ty][tx] = S;
    __syncthreads();
    S = part[0][tx];
#pragma unroll
    for (int w = 1; w < 8; ++w) S = max(S, part[w][tx]);
    if (ty == 0 && n < N) exps[n] = S;
    const float sc = pow2f_safe(-S);
    for (int k0 = 0; k0 < Kp; k0 += 64) {
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int kk = ty * 8 + j, k = k0 + kk;
            float2 v = make_float2(0.f, 0.f);
            if (n < N && k < K && S > -1000) v = src[(long long)k * ld + n];
            __nv_bfloat16 d[NS];
            ff_digits<NS>(v.x * sc, v.y * sc, d);
#pragma unroll
            for (int t = 0; t < NS; ++t) tile[t][tx][kk] = d[t];
        }
        __syncthreads();
        // warp ty writes rows 4ty..4ty+3 of the strip, 64 k = 128 bytes per row
        const int kw = k0 + 2 * tx;
#pragma unroll
        for (int t = 0; t < NS; ++t)
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const int nn = ty * 4 + rr;
                const long long col = n0 + nn;
                if (col < N && kw < Kp) {
                    uint32_t w = pack_bf16x2(tile[t][nn][2 * tx], tile[t][nn][2 * tx + 1]);
                    *reinterpret_cast<uint32_t*>(out + ((long long)t * N + col) * Kp + kw) = w;
                }
            }
    }
}

template <class Src>
static void launch_slice_rows(int s, Src src, long long M, int K, int Kp, __nv_bfloat16* out,
                              int* exps, cudaStream_t st) {
    const unsigned g = (unsigned)std::min<long long>((M + 7) / 8, 152LL * 64);
    switch (s) {
        case 2: k_slice_rows<2><<<g, 256, 0, st>>>(src, M, K, Kp, out, exps); break;
        case 3: k_slice_rows<3><<<g, 256, 0, st>>>(src, M, K, Kp, out, exps); break;
        case 4: k_slice_rows<4><<<g, 256, 0, st>>>(src, M, K, Kp, out, exps); break;
        case 5: k_slice_rows<5><<<g, 256, 0, st>>>(src, M, K, Kp, out, exps); break;
        default: k_slice_rows<6><<<g, 256, 0, st>>>(src, M, K, Kp, out, exps); break;
    }
}

static void launch_slice_cols(int s, const float2* src, long long ld, int K, long long N, int Kp,
                              int* exps, __nv_bfloat16* out, cudaStream_t st) {
    const unsigned g = (unsigned)((N + 31) / 32);
    switch (s) {
        case 2: k_slice_cols<2><<<g, 256, 0, st>>>(src, ld, K, N, Kp, exps, out); break;
        case 3: k_slice_cols<3><<<g, 256, 0, st>>>(src, ld, K, N, Kp, exps, out); break;
        case 4: k_slice_cols<4><<<g, 256, 0, st>>>(src, ld, K, N, Kp, exps, out); break;
        case 5: k_slice_cols<5><<<g, 256, 0, st>>>(src, ld, K, N, Kp, exps, out); break;
        default: k_slice_cols<6><<<g, 256, 0, st>>>(src, ld, K, N, Kp, exps, out); break;
    }
}

// ---------------------------------------------------------------------------
// host-side slicing of the constant operands (same digit arithmetic)
// ---------------------------------------------------------------------------
static inline uint16_t host_bf16(float f) {  // exact for digits (<= 8 significant bits)
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (uint16_t)(u >> 16);
}

// A operand: rows of a row-major double matrix (M x K)
static void host_slice_rows(const std::vector<double>& a, int M, int K, int Kp, int s,
                            std::vector<uint16_t>& out, std::vector<int>& exps) {
    out.assign((size_t)s * M * Kp, 0);
    exps.assign(M, -2000);
    for (int i = 0; i < M; ++i) {
        int S = -2000;
        for (int k = 0; k < K; ++k) S = std::max(S, scale_exp_f64(a[(size_t)i * K + k], slicing_wide(K)));
        exps[i] = S;
        if (S < -1000) continue;
        for (int k = 0; k < K; ++k) {
            int d[MAX_SLICES + 1];
            digits7(fixed_f64(a[(size_t)i * K + k], S, s), s, d);
            for (int t = 0; t < s; ++t)
                out[((size_t)t * M + i) * Kp + k] = host_bf16(std::ldexp((float)d[t], -7 * (t - 1)));
        }
    }
}

// B operand: columns of a row-major double matrix (K x N), output [s][N][Kp]
static void host_slice_cols(const double* b, int K, int N, long long ld, int Kp, int s,
                            std::vector<uint16_t>& out, std::vector<int>& exps) {
    out.assign((size_t)s * N * Kp, 0);
    exps.assign(N, -2000);
    for (int j = 0; j < N; ++j) {
        int S = -2000;
        for (int k = 0; k < K; ++k) S = std::max(S, scale_exp_f64(b[(size_t)k * ld + j], slicing_wide(K)));
        exps[j] = S;
        if (S < -1000) continue;
        for (int k = 0; k < K; ++k) {
            int d[MAX_SLICES + 1];
            digits7(fixed_f64(b[(size_t)k * ld + j], S, s), s, d);
            for (int t = 0; t < s; ++t)
                out[((size_t)t * N + j) * Kp + k] = host_bf16(std::ldexp((float)d[t], -7 * (t - 1)));
        }
    }
}

// ---------------------------------------------------------------------------
// the tcgen05 GEMM
// ---------------------------------------------------------------------------
struct SplitArgs {
    long long M, N;
    int Kp, s;
    int tiles_m, tiles_n;
    // split-K: K block range [ks*kcb, (ks+1)*kcb) of split ks < ksplit, with
    // its own scales row_exp[ks*M + row], col_exp[ks*N + col]; the epilogue
    // writes split ks as rows ks*M + row (ksplit = 1: plain GEMM)
    int ksplit, kcb;
    const int* row_exp;
    const int* col_exp;
    int* error;
};

constexpr int EPI_WARPS = 8;                 // two per TMEM lane group
constexpr int EC = 16;                       // epilogue columns per TMEM load
constexpr int GEMM_THREADS = 64 + 32 * EPI_WARPS;

// Where the tiles of a launch come from.  One problem: the kernel
// parameters.  A group: tables in global memory (per problem its arguments,
// its two tensor maps and its epilogue, and the first global tile index).
template <class Epi>
struct OneProblem {
    const CUtensorMap* ma;
    const CUtensorMap* mb;
    SplitArgs g;
    Epi e;
    __device__ __forceinline__ long long ntiles() const {
        return (long long)g.tiles_m * g.tiles_n * g.ksplit;
    }
    __device__ __forceinline__ int find(long long) const { return 0; }
    __device__ __forceinline__ long long first(int) const { return 0; }
    __device__ __forceinline__ const SplitArgs& args(int) const { return g; }
    __device__ __forceinline__ const CUtensorMap* mapA(int) const { return ma; }
    __device__ __forceinline__ const CUtensorMap* mapB(int) const { return mb; }
    __device__ __forceinline__ const Epi& epi(int) const { return e; }
};

template <class Epi>
struct GroupTable {
    const SplitArgs* g;        // [nprob]
    const CUtensorMap* maps;   // [2 * nprob]: A, B (64-byte aligned)
    const Epi* e;              // [nprob]
    const long long* start;    // [nprob + 1]: first global tile of each problem
    int nprob;
    __device__ __forceinline__ long long ntiles() const { return start[nprob]; }
    __device__ __forceinline__ int find(long long t) const {
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (start[mid] <= t) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }
    __device__ __forceinline__ long long first(int p) const { return start[p]; }
    __device__ __forceinline__ const SplitArgs& args(int p) const { return g[p]; }
    __device__ __forceinline__ const CUtensorMap* mapA(int p) const { return maps + 2 * p; }
    __device__ __forceinline__ const CUtensorMap* mapB(int p) const { return maps + 2 * p + 1; }
    __device__ __forceinline__ Epi epi(int p) const { return e[p]; }
};

// tile t of a launch: problem, output tile (tm, tn), K split and K blocks
struct TileRef {
    int p, ks, kb0, kb1;
    long long tm, tn;
};

template <class Tab>
__device__ __forceinline__ TileRef tile_ref(const Tab& tab, long long t) {
    TileRef r;
    r.p = tab.find(t);
    const SplitArgs& g = tab.args(r.p);
    const long long l = t - tab.first(r.p);
    const long long tmn = l / g.ksplit;
    r.ks = (int)(l - tmn * g.ksplit);
    r.kb0 = r.ks * g.kcb;
    r.kb1 = min(g.Kp / SBK, r.kb0 + g.kcb);
    if (g.tiles_m < g.tiles_n) {
        // fewer row tiles: they vary fastest, so the CTAs that share a tile of
        // the large B operand run at the same time and read it once from DRAM
        r.tn = tmn / g.tiles_m;
        r.tm = tmn - r.tn * g.tiles_m;
        return r;
    }
    r.tm = tmn / g.tiles_n;
    r.tn = tmn - r.tm * g.tiles_n;
    return r;
}

// The digit products of one staged K block, unrolled for S slices: A slice
// t times B slice u for t + u < S into accumulator min(t + u, 3) (one exact
// sum per product diagonal, the rest together).  A tile's first K block
// overwrites each accumulator with its first product.  Descriptors advance
// through the stage by adding byte offsets / 16 to the start-address field
// (stage addresses stay below 2^18, so the 14-bit field does not carry).
template <int S, bool PAIR>
__device__ __forceinline__ void issue_digit_products(uint32_t tmem, uint32_t acc_cols, uint64_t da0, uint64_t db0,
                                                     uint32_t slice_a16, uint32_t slice_b16, uint32_t idesc,
                                                     bool first) {
#pragma unroll
    for (int t = 0; t < S; ++t)
#pragma unroll
        for (int u = 0; u + t < S; ++u) {
            const uint32_t dt = tmem + (uint32_t)(t + u < 3 ? t + u : 3) * acc_cols;
            const uint64_t da = da0 + (uint64_t)(t * slice_a16), db = db0 + (uint64_t)(u * slice_b16);
#pragma unroll
            for (int kk = 0; kk < SBK / 16; ++kk) {
                const uint32_t accumulate = (first && t == 0 && kk == 0 && u <= 3) ? 0u : 1u;
                if (PAIR)
                    umma_bf16_pair(dt, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, accumulate);
                else
                    umma_bf16(dt, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, accumulate);
            }
        }
}

template <bool PAIR>
__device__ __forceinline__ void issue_stage(int s, uint32_t tmem, uint32_t acc_cols, uint64_t da0, uint64_t db0,
                                            uint32_t slice_a16, uint32_t slice_b16, uint32_t idesc, bool first) {
    switch (s) {
        case 1: issue_digit_products<1, PAIR>(tmem, acc_cols, da0, db0, slice_a16, slice_b16, idesc, first); break;
        case 2: issue_digit_products<2, PAIR>(tmem, acc_cols, da0, db0, slice_a16, slice_b16, idesc, first); break;
        case 3: issue_digit_products<3, PAIR>(tmem, acc_cols, da0, db0, slice_a16, slice_b16, idesc, first); break;
        case 4: issue_digit_products<4, PAIR>(tmem, acc_cols, da0, db0, slice_a16, slice_b16, idesc, first); break;
        case 5: issue_digit_products<5, PAIR>(tmem, acc_cols, da0, db0, slice_a16, slice_b16, idesc, first); break;
        default: issue_digit_products<6, PAIR>(tmem, acc_cols, da0, db0, slice_a16, slice_b16, idesc, first); break;
    }
}

// The GEMM body: BN = output tile width (128 or 64), s slices.
template <int BN, class Epi, class Tab>
__device__ __forceinline__ void split_gemm_body(const Tab& tab, int s, int* error,
                                                unsigned long long wait_ns = WAIT_NS,
                                                bool no_copies = false) {
    constexpr uint32_t TCOLS = 4 * BN;  // four accumulators of BN columns
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[NSTAGE], empty[NSTAGE], tfull, tempty, tdrain;
    __shared__ uint32_t tbase;
    __shared__ volatile int abort_flag;
    __shared__ int issued[NSTAGE];
    __shared__ float fcol_w[EPI_WARPS][BN / 2];  // per epilogue warp: 2^ecol of its columns
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t slice_a = SBM * SBK * 2, slice_b = BN * SBK * 2;
    const uint32_t stage_bytes = (uint32_t)s * (slice_a + slice_b);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long ntiles = tab.ntiles();
    if (threadIdx.x == 0) {
        for (int i = 0; i < NSTAGE; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
            issued[i] = 0;
        }
        mbar_init(&tfull, 1);
        mbar_init(&tempty, EPI_WARPS);
        mbar_init(&tdrain, 1);
        abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc(&tbase, TCOLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tbase;

    if (warp == 0) {
        if (lane == 0) {  // ---- TMA producer ----
            long long gk = 0;
            for (long long tile = blockIdx.x; tile < ntiles && !abort_flag; tile += gridDim.x) {
                const TileRef r = tile_ref(tab, tile);
                const SplitArgs& g = tab.args(r.p);
                const CUtensorMap* ma = tab.mapA(r.p);
                const CUtensorMap* mb = tab.mapB(r.p);
                for (int kb = r.kb0; kb < r.kb1; ++kb, ++gk) {
                    const int st = (int)(gk % NSTAGE);
                    const uint32_t ph = (uint32_t)((gk / NSTAGE) & 1);
                    if (!mbar_wait_bounded(&empty[st], ph ^ 1u, &abort_flag, wait_ns)) {
                        if (!abort_flag) atomicCAS(error, 0, ERR_TIMEOUT_EMPTY);
                        abort_flag = 1;
                        break;
                    }
                    unsigned char* base = smem + (size_t)st * stage_bytes;
                    mbar_expect_tx(&full[st], stage_bytes);
                    if (no_copies) continue;  // test hook: the MMA waits then run out
                    // all s slices of each operand tile in one 3D box
                    tma_load_3d(base, ma, &full[st], kb * SBK, (int)(r.tm * SBM), 0);
                    tma_load_3d(base + (size_t)s * slice_a, mb, &full[st], kb * SBK,
                                (int)(r.tn * BN), 0);

                    issued[st] = 1 + (int)ph;  // phase parity of the outstanding load
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // ---- MMA issuer ----
            const uint32_t idesc = umma_idesc_bf16(SBM, BN);
            long long gk = 0;
            int it = 0;
            for (long long tile = blockIdx.x; tile < ntiles && !abort_flag; tile += gridDim.x, ++it) {
                if (it > 0 && !mbar_wait_bounded(&tempty, (uint32_t)((it - 1) & 1), &abort_flag, wait_ns)) {
                    if (!abort_flag) atomicCAS(error, 0, ERR_TIMEOUT_TMEM);
                    abort_flag = 1;
                    break;
                }
                tc_fence_after();
                const TileRef r = tile_ref(tab, tile);
                for (int kb = r.kb0; kb < r.kb1; ++kb, ++gk) {
                    const int st = (int)(gk % NSTAGE);
                    const uint32_t ph = (uint32_t)((gk / NSTAGE) & 1);
                    if (!mbar_wait_bounded(&full[st], ph, &abort_flag, wait_ns)) {
                        if (!abort_flag) atomicCAS(error, 0, ERR_TIMEOUT_FULL);
                        abort_flag = 1;
                        break;
                    }
                    issued[st] = 0;
                    tc_fence_after();
                    unsigned char* base = smem + (size_t)st * stage_bytes;
                    issue_stage<false>(s, tmem, BN, umma_sdesc(base, 512, UMMA_SWIZZLE_64B),
                                       umma_sdesc(base + (size_t)s * slice_a, 512, UMMA_SWIZZLE_64B),
                                       slice_a >> 4, slice_b >> 4, idesc, kb == r.kb0);
                    umma_commit(&empty[st]);
                }
                if (abort_flag) break;
                umma_commit(&tfull);
            }
            // every MMA this thread issued completes before TMEM is freed
            // (after an abort, the last ones were never waited for)
            umma_commit(&tdrain);
            volatile int never = 0;
            if (!mbar_wait_bounded(&tdrain, 0, &never, WAIT_NS)) atomicOr(error, ERR_DRAIN_UNCONFIRMED);
        }
    } else {  // ---- epilogue: warps 2..9; lane group warp%4, column half (warp-2)/4 ----
        const int ew = warp - 2;
        const int lg = warp & 3;
        const int chalf = ew >> 2;
        const uint32_t lane_base = (uint32_t)(lg * 32) << 16;
        int it = 0;
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
            // the whole warp leaves together (the TMEM loads and __syncwarp
            // below need every lane)
            if (__any_sync(0xffffffffu, abort_flag != 0)) break;
            const TileRef r = tile_ref(tab, tile);
            const SplitArgs& g = tab.args(r.p);
            const long long ks = r.ks, tm = r.tm, tn = r.tn;
            // column scale factors of this warp's half tile (warp-local: no
            // barrier another role could leave waiting)
            float* fcol = fcol_w[ew];
            __syncwarp();
            for (int j = lane; j < BN / 2; j += 32) {
                const long long col = tn * BN + chalf * (BN / 2) + j;
                const int e = col < g.N ? g.col_exp[ks * g.N + col] : -2000;
                fcol[j] = e < -1000 ? 0.0f : pow2f_safe(e);
            }
            __syncwarp();
            const bool ready = __all_sync(
                0xffffffffu, mbar_wait_bounded(&tfull, (uint32_t)(it & 1), &abort_flag, wait_ns));
            if (!ready) {
                if (lane == 0 && !abort_flag) atomicCAS(error, 0, ERR_TIMEOUT_TMEM);
                abort_flag = 1;
                break;
            }
            tc_fence_after();
            const long long row = tm * SBM + lg * 32 + lane;
            const int erow = row < g.M ? g.row_exp[ks * g.M + row] : -2000;
            const float frow = erow < -1000 ? 0.0f : pow2f_safe(erow - 28);
            const auto& epi = tab.epi(r.p);
            const typename Epi::Row er = epi.row(ks * g.M + (row < g.M ? row : 0));
            for (int c0 = chalf * (BN / 2); c0 < (chalf + 1) * (BN / 2); c0 += EC) {
                uint32_t r0[EC], r1[EC], r2[EC], r3[EC];
                tmem_ld16(tmem + lane_base + (uint32_t)c0, r0);
                if (s >= 2) tmem_ld16(tmem + lane_base + (uint32_t)(BN + c0), r1);
                if (s >= 3) tmem_ld16(tmem + lane_base + (uint32_t)(2 * BN + c0), r2);
                if (s >= 4) tmem_ld16(tmem + lane_base + (uint32_t)(3 * BN + c0), r3);
                tmem_ld_wait();
                if (c0 + EC == (chalf + 1) * (BN / 2)) {  // this warp's accumulators drained
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty);
                }
                if (row >= g.M) continue;
#pragma unroll
                for (int j = 0; j < EC; ++j) {
                    const float a0 = __uint_as_float(r0[j]);
                    const float a1 = s >= 2 ? __uint_as_float(r1[j]) : 0.f;
                    const float a2 = s >= 3 ? __uint_as_float(r2[j]) : 0.f;
                    const float a3 = s >= 4 ? __uint_as_float(r3[j]) : 0.f;
                    // exact sum of the exact diagonals, then the rounded tail
                    float s1, e1, s2, e2, s3, e3, hi, lo;
                    two_sum(a0, a1, s1, e1);
                    two_sum(s1, a2, s2, e2);
                    two_sum(s2, a3, s3, e3);
                    fast_two_sum(s3, (e1 + e2) + e3, hi, lo);
                    const float f = fcol[c0 - chalf * (BN / 2) + j] * frow;  // 2^(erow+ecol-28)
                    r0[j] = __float_as_uint(hi * f);   // the accumulator registers now hold
                    r1[j] = __float_as_uint(lo * f);   // the float-float result
                }
                epi.store(er, tn * BN + c0, g.N, r0, r1);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && abort_flag) {
        // let the outstanding tensor copies of this CTA land before exit
        volatile int never = 0;
        for (int st = 0; st < NSTAGE; ++st)
            if (issued[st] && !mbar_wait_bounded(&full[st], (uint32_t)(issued[st] - 1), &never, WAIT_NS))
                atomicOr(error, ERR_COPIES_UNCONFIRMED);
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TCOLS);
}

// ---------------------------------------------------------------------------
// The CTA-pair GEMM: clusters of two CTAs, one 2-SM MMA (tcgen05.mma
// cta_group::2, M = 256, N = 128) issued by the even CTA.  Each CTA stages its
// 128 rows of A and half (64 columns) of B -- 12 KB per slice and K block
// instead of 16 KB -- so three pipeline stages fit, and the shared-memory
// fill per output element is 3/4 of the single-CTA kernel's.  Both CTAs'
// tensor copies count on the even CTA's full barriers; MMA completion is
// multicast to both CTAs' empty and accumulator barriers; each CTA drains its
// own TMEM lanes (its 128 rows) and signals the even CTA.
// ---------------------------------------------------------------------------
constexpr int PSTAGE = 3, PBM = 256, PBN = 128;

// The j-th tile of pair `pair` (npairs pairs).  One problem: the tiles of
// the shorter dimension are taken together (a strip), so the tile of the
// longer operand is read from DRAM once and then from L2 by the same pair.
template <class Epi>
__device__ __forceinline__ bool pair_next(const OneProblem<Epi>& tab, long long pair, long long j,
                                          long long npairs, TileRef& r) {
    const SplitArgs& g = tab.g;
    const bool mshort = g.tiles_m <= g.tiles_n;
    const long long U = mshort ? g.tiles_m : g.tiles_n, L = mshort ? g.tiles_n : g.tiles_m;
    const long long strip = pair + (j / U) * npairs;
    if (strip >= L) return false;
    const long long inner = j - (j / U) * U;
    r.p = 0;
    r.ks = 0;
    r.kb0 = 0;
    r.kb1 = g.Kp / SBK;
    r.tm = mshort ? inner : strip;
    r.tn = mshort ? strip : inner;
    return true;
}

template <class Epi, class Tab>
__device__ __forceinline__ void split_gemm_pair_body(const Tab& tab, int s, int* error,
                                                     unsigned long long wait_ns, bool no_copies) {
    constexpr uint32_t TCOLS = 4 * PBN;  // four accumulators of 128 columns
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t full[PSTAGE], empty[PSTAGE], tfull, tempty, tdrain;
    __shared__ uint32_t tbase;
    __shared__ volatile int abort_flag;
    __shared__ float fcol_w[EPI_WARPS][PBN / 2];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t slice_a = (PBM / 2) * SBK * 2, slice_b = (PBN / 2) * SBK * 2;
    const uint32_t stage_bytes = (uint32_t)s * (slice_a + slice_b);  // per CTA
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_ctarank();
    const long long pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;
    if (threadIdx.x == 0) {
        for (int i = 0; i < PSTAGE; ++i) {
            mbar_init(&full[i], 1);   // the even CTA's producer (expects both CTAs' bytes)
            mbar_init(&empty[i], 1);  // one multicast MMA commit per use of the stage
        }
        mbar_init(&tfull, 1);
        mbar_init(&tempty, 2 * EPI_WARPS);  // the epilogue warps of both CTAs
        mbar_init(&tdrain, 1);
        abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) tmem_alloc_pair(&tbase, TCOLS);
    tc_fence_before();
    cluster_sync();  // barriers of both CTAs initialised, TMEM allocated
    tc_fence_after();
    const uint32_t tmem = tbase;
    const uint32_t abort_peer = mapa_shared(smem_u32((const void*)&abort_flag), rank ^ 1u);
    // give up: record the first cause, stop both CTAs' roles
    auto give_up = [&](int code) {
        if (!abort_flag) atomicCAS(error, 0, code);
        abort_flag = 1;
        st_cluster_u32(abort_peer, 1u);
    };

    if (warp == 0) {
        if (lane == 0) {  // ---- TMA producer (both CTAs) ----
            uint32_t fullc[PSTAGE];
            for (int i = 0; i < PSTAGE; ++i) fullc[i] = mapa_shared(smem_u32(&full[i]), 0);
            long long gk = 0;
            TileRef r;
            for (long long j = 0; !abort_flag && pair_next(tab, pair, j, npairs, r); ++j) {
                const CUtensorMap* ma = tab.mapA(r.p);
                const CUtensorMap* mb = tab.mapB(r.p);
                for (int kb = r.kb0; kb < r.kb1; ++kb, ++gk) {
                    const int st = (int)(gk % PSTAGE);
                    const uint32_t ph = (uint32_t)((gk / PSTAGE) & 1);
                    if (!mbar_wait_bounded(&empty[st], ph ^ 1u, &abort_flag, wait_ns)) {
                        if (!abort_flag) give_up(ERR_TIMEOUT_EMPTY);
                        break;
                    }
                    if (rank == 0) mbar_expect_tx(&full[st], 2 * stage_bytes);
                    if (no_copies) continue;  // test hook: the MMA waits then run out
                    unsigned char* base = smem + (size_t)st * stage_bytes;
                    tma_load_3d_pair(base, ma, fullc[st], kb * SBK, (int)(r.tm * PBM + rank * (PBM / 2)), 0);
                    tma_load_3d_pair(base + (size_t)s * slice_a, mb, fullc[st], kb * SBK,
                                     (int)(r.tn * PBN + rank * (PBN / 2)), 0);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {  // ---- MMA issuer (even CTA) ----
            const uint32_t idesc = umma_idesc_bf16(PBM, PBN);
            long long gk = 0;
            int it = 0;
            TileRef r;
            for (long long j = 0; !abort_flag && pair_next(tab, pair, j, npairs, r); ++j, ++it) {
                if (it > 0 && !mbar_wait_bounded(&tempty, (uint32_t)((it - 1) & 1), &abort_flag, wait_ns)) {
                    if (!abort_flag) give_up(ERR_TIMEOUT_TMEM);
                    break;
                }
                tc_fence_after();
                for (int kb = r.kb0; kb < r.kb1; ++kb, ++gk) {
                    const int st = (int)(gk % PSTAGE);
                    const uint32_t ph = (uint32_t)((gk / PSTAGE) & 1);
                    if (!mbar_wait_bounded(&full[st], ph, &abort_flag, wait_ns)) {
                        if (!abort_flag) give_up(ERR_TIMEOUT_FULL);
                        break;
                    }
                    tc_fence_after();
                    unsigned char* base = smem + (size_t)st * stage_bytes;
                    issue_stage<true>(s, tmem, PBN, umma_sdesc(base, 512, UMMA_SWIZZLE_64B),
                                      umma_sdesc(base + (size_t)s * slice_a, 512, UMMA_SWIZZLE_64B),
                                      slice_a >> 4, slice_b >> 4, idesc, kb == r.kb0);
                    umma_commit_pair(&empty[st], (uint16_t)3);
                }
                if (abort_flag) break;
                umma_commit_pair(&tfull, (uint16_t)3);
            }
            // every MMA issued completes before TMEM is freed
            umma_commit_pair(&tdrain, (uint16_t)1);
            volatile int never = 0;
            if (!mbar_wait_bounded(&tdrain, 0, &never, WAIT_NS)) atomicOr(error, ERR_DRAIN_UNCONFIRMED);
        }
    } else {  // ---- epilogue: warps 2..9 of both CTAs; lane group warp%4, column half (warp-2)/4 ----
        const int ew = warp - 2;
        const int lg = warp & 3;
        const int chalf = ew >> 2;
        const uint32_t lane_base = (uint32_t)(lg * 32) << 16;
        const uint32_t tempty0 = mapa_shared(smem_u32(&tempty), 0);
        int it = 0;
        TileRef r;
        for (long long j = 0; pair_next(tab, pair, j, npairs, r); ++j, ++it) {
            if (__any_sync(0xffffffffu, abort_flag != 0)) break;
            const SplitArgs& g = tab.args(r.p);
            const long long ks = r.ks, tm = r.tm, tn = r.tn;
            float* fcol = fcol_w[ew];
            __syncwarp();
            for (int jj = lane; jj < PBN / 2; jj += 32) {
                const long long col = tn * PBN + chalf * (PBN / 2) + jj;
                const int e = col < g.N ? g.col_exp[ks * g.N + col] : -2000;
                fcol[jj] = e < -1000 ? 0.0f : pow2f_safe(e);
            }
            __syncwarp();
            const bool ready = __all_sync(
                0xffffffffu, mbar_wait_bounded(&tfull, (uint32_t)(it & 1), &abort_flag, wait_ns));
            if (!ready) {
                if (lane == 0) give_up(ERR_TIMEOUT_TMEM);
                break;
            }
            tc_fence_after();
            const long long row = tm * PBM + rank * (PBM / 2) + lg * 32 + lane;
            const int erow = row < g.M ? g.row_exp[ks * g.M + row] : -2000;
            const float frow = erow < -1000 ? 0.0f : pow2f_safe(erow - 28);
            const auto& epi = tab.epi(r.p);
            const typename Epi::Row er = epi.row(ks * g.M + (row < g.M ? row : 0));
            for (int c0 = chalf * (PBN / 2); c0 < (chalf + 1) * (PBN / 2); c0 += EC) {
                uint32_t r0[EC], r1[EC], r2[EC], r3[EC];
                tmem_ld16(tmem + lane_base + (uint32_t)c0, r0);
                if (s >= 2) tmem_ld16(tmem + lane_base + (uint32_t)(PBN + c0), r1);
                if (s >= 3) tmem_ld16(tmem + lane_base + (uint32_t)(2 * PBN + c0), r2);
                if (s >= 4) tmem_ld16(tmem + lane_base + (uint32_t)(3 * PBN + c0), r3);
                tmem_ld_wait();
                if (c0 + EC == (chalf + 1) * (PBN / 2)) {  // this warp's accumulators drained
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive_cluster(tempty0);
                }
                if (row >= g.M) continue;
#pragma unroll
                for (int jj = 0; jj < EC; ++jj) {
                    const float a0 = __uint_as_float(r0[jj]);
                    const float a1 = s >= 2 ? __uint_as_float(r1[jj]) : 0.f;
                    const float a2 = s >= 3 ? __uint_as_float(r2[jj]) : 0.f;
                    const float a3 = s >= 4 ? __uint_as_float(r3[jj]) : 0.f;
                    float s1, e1, s2, e2, s3, e3, hi, lo;
                    two_sum(a0, a1, s1, e1);
                    two_sum(s1, a2, s2, e2);
                    two_sum(s2, a3, s3, e3);
                    fast_two_sum(s3, (e1 + e2) + e3, hi, lo);
                    const float f = fcol[c0 - chalf * (PBN / 2) + jj] * frow;  // 2^(erow+ecol-28)
                    r0[jj] = __float_as_uint(hi * f);
                    r1[jj] = __float_as_uint(lo * f);
                }
                epi.store(er, tn * PBN + c0, g.N, r0, r1);
            }
        }
    }
    // Both CTAs meet before either frees TMEM or leaves: no CTA exits while
    // the other can still write its shared memory or barriers.  After an
    // abort (every wait above is bounded, so both get here), tensor copies
    // either CTA issued may still be landing; their completion counts on the
    // even CTA's barriers, which an aborted pipeline may never complete, so
    // the CTA waits a fixed 1 ms -- far longer than a copy takes.
    tc_fence_before();
    cluster_sync();
    if (abort_flag && threadIdx.x == 0) {
        const unsigned long long t0 = global_ns();
        while (global_ns() - t0 < 1000000ull) {
        }
    }
    cluster_sync();
    tc_fence_after();
    __syncwarp();
    if (warp == 0) tmem_dealloc_pair(tmem, TCOLS);
}

template <class Epi>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(GEMM_THREADS, 1)
    k_split_gemm_pair(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                      SplitArgs g, Epi epi, unsigned long long wait_ns, int no_copies) {
    const OneProblem<Epi> tab{&mapA, &mapB, g, epi};
    split_gemm_pair_body<Epi>(tab, g.s, g.error, wait_ns, no_copies != 0);
}

// One problem: operands through kernel-parameter tensor maps.
template <int BN, class Epi>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_split_gemm(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                 SplitArgs g, Epi epi, unsigned long long wait_ns, int no_copies) {
    const OneProblem<Epi> tab{&mapA, &mapB, g, epi};
    split_gemm_body<BN, Epi>(tab, g.s, g.error, wait_ns, no_copies != 0);
}

// A group of problems (one persistent launch over all their tiles).
template <int BN, class Epi>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    k_split_gemm_grouped(GroupTable<Epi> tab, int s, int* error) {
    split_gemm_body<BN, Epi>(tab, s, error);
}

// ---------------------------------------------------------------------------
// epilogue functors (float-float outputs)
// ---------------------------------------------------------------------------
// Each functor maps an output row once (row()) and then stores EC
// consecutive columns col0.. of it (store(), columns >= N skipped).
struct EpiFF_HA {  // GEMM1: row = r*npc + pql, col = plane*m + b -> HA[plane][r0+r][b][pql]
    float2* ha;
    int r0, m, npc;
    long long plane;
    typedef float2* Row;
    __device__ __forceinline__ Row row(long long i) const {
        const long long r = i / npc, q = i - r * npc;
        return ha + (r0 + r) * (long long)m * npc + q;
    }
    __device__ __forceinline__ void store(Row p, long long col0, long long N, const uint32_t (&h)[EC],
                                         const uint32_t (&l)[EC]) const {
#pragma unroll
        for (int j = 0; j < EC; ++j) {
            const long long col = col0 + j;
            if (col >= N) break;
            const int pl = col >= m;
            p[pl * plane + (col - pl * m) * npc] = make_float2(__uint_as_float(h[j]), __uint_as_float(l[j]));
        }
    }
};

struct EpiFF_RowMajor {  // C[row][col], leading dimension ldc
    float2* c;
    long long ldc;
    // optional row map: with rblk > 0, row i is output row
    // (i / rblk) * mrow + rblk + i % rblk (the barred half of each plane);
    // columns start at col_off
    long long rblk = 0, mrow = 0, col_off = 0;
    typedef float2* Row;
    __device__ __forceinline__ Row row(long long i) const {
        const long long r = rblk ? (i / rblk) * mrow + rblk + i % rblk : i;
        return c + r * ldc + col_off;
    }
    __device__ __forceinline__ void store(Row p, long long col0, long long N, const uint32_t (&h)[EC],
                                         const uint32_t (&l)[EC]) const {
        if (col0 + EC <= N && (((uintptr_t)(p + col0)) & 15) == 0) {
#pragma unroll
            for (int j = 0; j < EC; j += 2)
                *reinterpret_cast<uint4*>(p + col0 + j) = make_uint4(h[j], l[j], h[j + 1], l[j + 1]);
        } else {
#pragma unroll
            for (int j = 0; j < EC; ++j)
                if (col0 + j < N) p[col0 + j] = make_float2(__uint_as_float(h[j]), __uint_as_float(l[j]));
        }
    }
};

struct EpiFF_RK {  // GEMM3: row = (p, ijl), col = plane*m + k -> RK[plane][c0+p][ijl][k]
    float2* rk;
    int m;
    long long rowoff, plane;
    typedef float2* Row;
    __device__ __forceinline__ Row row(long long i) const { return rk + (rowoff + i) * m; }
    __device__ __forceinline__ void store(Row p, long long col0, long long N, const uint32_t (&h)[EC],
                                         const uint32_t (&l)[EC]) const {
#pragma unroll
        for (int j = 0; j < EC; ++j) {
            const long long col = col0 + j;
            if (col >= N) break;
            const int pl = col >= m;
            p[pl * plane + (col - pl * m)] = make_float2(__uint_as_float(h[j]), __uint_as_float(l[j]));
        }
    }
};

struct EpiF64_RowMajor {  // C[row][col] = hi + lo rounded to FP64, leading dimension ldc
    double* c;
    long long ldc;
    typedef double* Row;
    __device__ __forceinline__ Row row(long long i) const { return c + i * ldc; }
    __device__ __forceinline__ void store(Row p, long long col0, long long N, const uint32_t (&h)[EC],
                                         const uint32_t (&l)[EC]) const {
#pragma unroll
        for (int j = 0; j < EC; ++j)
            if (col0 + j < N)
                p[col0 + j] = (double)__uint_as_float(h[j]) + (double)__uint_as_float(l[j]);
    }
};

// ---------------------------------------------------------------------------
// state and host orchestration
// ---------------------------------------------------------------------------
struct ConstSlices {
    __nv_bfloat16* d = nullptr;
    int* exps = nullptr;
    int rows = 0, K = 0, Kp = 0;
};

struct SplitState {
    int s = 6;
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    int num_sms = 152;
    int max_pairs = 0;  // CTA pairs of the pair kernel resident at once
    bool use_pairs = false;  // RT_GEMM_KERNEL=pair selects the CTA-pair kernel for M > 128
    // constant operands
    ConstSlices qah;                 // A of GEMM2/4: rows 2m, K = 2n
    ConstSlices qahB;                // the barred rows of qah (both planes): rows m
    std::vector<ConstSlices> qap;    // B of GEMM1 per AO block: N = 2m, K = block size
    ConstSlices qar[2];              // B of GEMM3 per component: N = 2m, K = 2nc
    ConstSlices qc[2];               // B of the adjoint's X GEMM per component: N = 2m, K = nc
    // Gaunt (Breit) transformation: the operands built from QB
    ConstSlices qbh;                 // A of GEMM4 for the third stream: rows 2m, K = 2n
    ConstSlices qbhS;                // A of the QB^H HA GEMM (large-component columns zero)
    ConstSlices qbr[2];              // B of GEMM3 for the second stream, per component
    // work buffers
    __nv_bfloat16* a_sl = nullptr;
    int* a_exp = nullptr;
    size_t a_cap = 0, a_exp_cap = 0;
    __nv_bfloat16* b_sl = nullptr;
    int* b_exp = nullptr;
    size_t b_cap = 0, b_exp_cap = 0;
    int* d_err = nullptr;
    std::vector<void*> allocs;
};

static int kpad(int K) { return (K + SBK - 1) / SBK * SBK; }

// dynamic shared memory of the pair kernel: PSTAGE stages of s slices of a
// 128-row A tile and a 64-column B tile, plus the 1024-byte alignment slack
static size_t pair_smem_bytes(int s) {
    return (size_t)PSTAGE * s * (PBM / 2 + PBN / 2) * SBK * 2 + 1024;
}

// Clusters of two CTAs of a pair kernel that can be resident together (a
// persistent grid larger than that would run a second wave).
static int pair_capacity(const void* kernel, size_t smem, int num_sms) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(num_sms & ~1), 1, 1);
    cfg.blockDim = dim3(GEMM_THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) != cudaSuccess || n < 1) {
        cudaGetLastError();
        throw Error(RT_ERR_PROGRAM, "no CTA pair of the split GEMM fits on this device");
    }
    return std::min(n, num_sms / 2);
}

// Test hook for the GEMM's abort path: with RT_TEST_GEMM_NO_COPIES=1 in the
// environment a launch issues no tensor copies and gives its waits 50 ms, so
// the waits run out, the kernel stops all its roles and reports status 2
// (class 6 on the host) without faulting; the context stays usable.
static bool test_no_copies() {
    const char* e = getenv("RT_TEST_GEMM_NO_COPIES");
    return e && e[0] == '1';
}

static void* salloc(SplitState* S, size_t bytes) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(RT_ERR_DIM, std::string("split-path allocation failed: ") + cudaGetErrorString(e));
    }
    S->allocs.push_back(p);
    return p;
}

static void sfree(SplitState* S, void* p) {
    if (!p) return;
    auto it = std::find(S->allocs.begin(), S->allocs.end(), p);
    if (it != S->allocs.end()) S->allocs.erase(it);
    cudaFree(p);
}

template <class K>
static void set_smem_limit(K kernel, size_t need, const cudaDeviceProp& prop) {
    cudaFuncAttributes fa;
    RT_CUDA(cudaFuncGetAttributes(&fa, kernel));
    if (need + fa.sharedSizeBytes > prop.sharedMemPerBlockOptin)
        throw Error(RT_ERR_DIM, "split GEMM stages exceed the shared memory of one SM");
    RT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need));
}

static SplitState* state(rt_ctx* c) {
    if (!c->split) {
        SplitState* S = new SplitState();
        S->s = c->cfg.slices;
        if (S->s > MAX_SLICES) throw Error(RT_ERR_DIM, "at most 6 slices are supported");
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        RT_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                 cudaEnableDefault, &q));
        if (!fn || q != cudaDriverEntryPointSuccess)
            throw Error(RT_ERR_PROGRAM, "cuTensorMapEncodeTiled unavailable");
        S->encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
        cudaDeviceProp prop;
        RT_CUDA(cudaGetDeviceProperties(&prop, c->device));
        S->num_sms = prop.multiProcessorCount;
        S->d_err = (int*)salloc(S, sizeof(int));
        RT_CUDA(cudaMemset(S->d_err, 0, sizeof(int)));
        const size_t need = (size_t)NSTAGE * S->s * (SBM + SBN) * SBK * 2 + 1024;
        set_smem_limit(k_split_gemm<128, EpiFF_HA>, need, prop);
        set_smem_limit(k_split_gemm<128, EpiFF_RowMajor>, need, prop);
        set_smem_limit(k_split_gemm<128, EpiFF_RK>, need, prop);
        const size_t need2 = pair_smem_bytes(S->s);
        set_smem_limit(k_split_gemm_pair<EpiFF_HA>, need2, prop);
        set_smem_limit(k_split_gemm_pair<EpiFF_RowMajor>, need2, prop);
        set_smem_limit(k_split_gemm_pair<EpiFF_RK>, need2, prop);
        S->max_pairs = pair_capacity((const void*)k_split_gemm_pair<EpiFF_RowMajor>, need2, S->num_sms);
        // Choice between the two implementations of the same product
        // (identical digit arithmetic and accumulation): the single-CTA
        // kernel (default; measured faster on GB300 for these shapes) or,
        // with RT_GEMM_KERNEL=pair, the CTA-pair kernel for M > 128.
        const char* kv = getenv("RT_GEMM_KERNEL");
        S->use_pairs = kv && std::strcmp(kv, "pair") == 0;
        const char* tr = getenv("RT_TRACE");
        if (tr && std::strcmp(tr, "0") != 0)
            std::fprintf(stderr, "[rt] split GEMM: %s kernel, %d CTA pairs resident (%d SMs)\n",
                         S->use_pairs ? "CTA-pair" : "single-CTA", S->max_pairs, S->num_sms);
        c->split = S;
    }
    return c->split;
}

static void upload_const(SplitState* S, ConstSlices& cs, const std::vector<uint16_t>& sl,
                         const std::vector<int>& ex, int rows, int K) {
    sfree(S, cs.d);
    sfree(S, cs.exps);
    cs.d = (__nv_bfloat16*)salloc(S, sl.size() * 2);
    cs.exps = (int*)salloc(S, ex.size() * sizeof(int));
    RT_CUDA(cudaMemcpy(cs.d, sl.data(), sl.size() * 2, cudaMemcpyHostToDevice));
    RT_CUDA(cudaMemcpy(cs.exps, ex.data(), ex.size() * sizeof(int), cudaMemcpyHostToDevice));
    cs.rows = rows;
    cs.K = K;
    cs.Kp = kpad(K);
}

void split_prepare_constants(rt_ctx* c) {
    SplitState* S = state(c);
    const Plan& P = c->plan;
    const int n = P.n, m = P.m, s = S->s;
    if (2 * n > KMAX_EXACT)
        throw Error(RT_ERR_DIM, "split path: 2*NSC > " + std::to_string(KMAX_EXACT) +
                                    " exceeds the exact FP32 accumulation range");
    // planar QA in sorted AO order
    std::vector<double> qr((size_t)n * m), qi((size_t)n * m);
    for (int p = 0; p < n; ++p)
        for (int i = 0; i < m; ++i) {
            qr[(size_t)P.ao_sorted[p] * m + i] = c->qa[2 * ((size_t)p + (size_t)i * n)];
            qi[(size_t)P.ao_sorted[p] * m + i] = c->qa[2 * ((size_t)p + (size_t)i * n) + 1];
        }
    std::vector<uint16_t> sl;
    std::vector<int> ex;
    // qah: [(plane',a)][(plane,r)] rows 2m, K 2n
    {
        std::vector<double> a((size_t)2 * m * 2 * n);
        for (int i = 0; i < m; ++i)
            for (int r = 0; r < n; ++r) {
                double re = qr[(size_t)r * m + i], im = qi[(size_t)r * m + i];
                a[(size_t)i * 2 * n + r] = re;
                a[(size_t)i * 2 * n + n + r] = im;
                a[(size_t)(m + i) * 2 * n + r] = -im;
                a[(size_t)(m + i) * 2 * n + n + r] = re;
            }
        host_slice_rows(a, 2 * m, 2 * n, kpad(2 * n), s, sl, ex);
        upload_const(S, S->qah, sl, ex, 2 * m, 2 * n);
        // rows (plane, x) with x in the barred half [m/2, m) of the internal order
        const int K = m / 2;
        std::vector<double> ab((size_t)m * 2 * n);
        for (int pl = 0; pl < 2; ++pl)
            for (int j = 0; j < K; ++j)
                std::memcpy(&ab[((size_t)pl * K + j) * 2 * n], &a[((size_t)pl * m + K + j) * 2 * n],
                            sizeof(double) * 2 * n);
        host_slice_rows(ab, m, 2 * n, kpad(2 * n), s, sl, ex);
        upload_const(S, S->qahB, sl, ex, m, 2 * n);
    }
    // qap per AO block: B = rows s in block, cols (plane, b)
    S->qap.resize(P.nblk);
    for (int b = 0; b < P.nblk; ++b) {
        const int nk = P.blk_size[b], st = P.blk_start[b];
        std::vector<double> bm((size_t)nk * 2 * m);
        for (int k = 0; k < nk; ++k)
            for (int j = 0; j < m; ++j) {
                bm[(size_t)k * 2 * m + j] = qr[(size_t)(st + k) * m + j];
                bm[(size_t)k * 2 * m + m + j] = qi[(size_t)(st + k) * m + j];
            }
        host_slice_cols(bm.data(), nk, 2 * m, 2 * m, kpad(nk), s, sl, ex);
        upload_const(S, S->qap[b], sl, ex, 2 * m, nk);
    }
    // qar per component: [(plane,q)][(plane',k)] = [[QAr, QAi], [-QAi, QAr]]
    for (int comp = 0; comp < 2; ++comp) {
        const int nc = P.ncomp[comp], off = P.comp_off[comp];
        if (nc == 0) continue;
        std::vector<double> bm((size_t)2 * nc * 2 * m);
        for (int q = 0; q < nc; ++q)
            for (int k = 0; k < m; ++k) {
                double re = qr[(size_t)(off + q) * m + k], im = qi[(size_t)(off + q) * m + k];
                bm[(size_t)q * 2 * m + k] = re;
                bm[(size_t)q * 2 * m + m + k] = im;
                bm[(size_t)(nc + q) * 2 * m + k] = -im;
                bm[(size_t)(nc + q) * 2 * m + m + k] = re;
            }
        host_slice_cols(bm.data(), 2 * nc, 2 * m, 2 * m, kpad(2 * nc), s, sl, ex);
        upload_const(S, S->qar[comp], sl, ex, 2 * m, 2 * nc);
        // [QAr | QAi] of the component (adjoint)
        std::vector<double> bc((size_t)nc * 2 * m);
        for (int q = 0; q < nc; ++q)
            for (int j = 0; j < m; ++j) {
                bc[(size_t)q * 2 * m + j] = qr[(size_t)(off + q) * m + j];
                bc[(size_t)q * 2 * m + m + j] = qi[(size_t)(off + q) * m + j];
            }
        host_slice_cols(bc.data(), nc, 2 * m, 2 * m, kpad(nc), s, sl, ex);
        upload_const(S, S->qc[comp], sl, ex, 2 * m, nc);
    }
    if (!c->cfg.breit) return;
    // QB in sorted AO order from QA (QB(j) = -conj(QA(jbar)) for unbarred j,
    // QB(jbar) = conj(QA(j)); internal spinor order)
    std::vector<double> br((size_t)n * m), bi((size_t)n * m);
    for (int i = 0; i < m; ++i) {
        const int t = c->itrmo[i], pi = std::abs(t) - 1;
        const double sg = t > 0 ? -1.0 : 1.0;
        for (int r = 0; r < n; ++r) {
            br[(size_t)r * m + i] = sg * qr[(size_t)r * m + pi];
            bi[(size_t)r * m + i] = -sg * qi[(size_t)r * m + pi];
        }
    }
    {
        std::vector<double> a((size_t)2 * m * 2 * n), as((size_t)2 * m * 2 * n, 0.0);
        for (int i = 0; i < m; ++i)
            for (int r = 0; r < n; ++r) {
                double re = br[(size_t)r * m + i], im = bi[(size_t)r * m + i];
                size_t x[4] = {(size_t)i * 2 * n + r, (size_t)i * 2 * n + n + r, (size_t)(m + i) * 2 * n + r,
                               (size_t)(m + i) * 2 * n + n + r};
                double v[4] = {re, im, -im, re};
                for (int t = 0; t < 4; ++t) {
                    a[x[t]] = v[t];
                    if (r >= P.nL) as[x[t]] = v[t];  // small-component rows of HA only
                }
            }
        host_slice_rows(a, 2 * m, 2 * n, kpad(2 * n), s, sl, ex);
        upload_const(S, S->qbh, sl, ex, 2 * m, 2 * n);
        host_slice_rows(as, 2 * m, 2 * n, kpad(2 * n), s, sl, ex);
        upload_const(S, S->qbhS, sl, ex, 2 * m, 2 * n);
    }
    for (int comp = 0; comp < 2; ++comp) {
        const int nc = P.ncomp[comp], off = P.comp_off[comp];
        if (nc == 0) continue;
        std::vector<double> bm((size_t)2 * nc * 2 * m);
        for (int q = 0; q < nc; ++q)
            for (int k = 0; k < m; ++k) {
                double re = br[(size_t)(off + q) * m + k], im = bi[(size_t)(off + q) * m + k];
                bm[(size_t)q * 2 * m + k] = re;
                bm[(size_t)q * 2 * m + m + k] = im;
                bm[(size_t)(nc + q) * 2 * m + k] = -im;
                bm[(size_t)(nc + q) * 2 * m + m + k] = re;
            }
        host_slice_cols(bm.data(), 2 * nc, 2 * m, 2 * m, kpad(2 * nc), s, sl, ex);
        upload_const(S, S->qbr[comp], sl, ex, 2 * m, 2 * nc);
    }
}

double split_stageA_bytes_per_pair(rt_ctx* c) {
    const Plan& P = c->plan;
    const int s = c->cfg.slices;
    long long a_pp = 0;  // GEMM1 operand slices of all groups of a pair group (BF16 elements)
    for (long long v : P.pg_a_pp) a_pp = std::max(a_pp, v);
    double a = 2.0 * a_pp;
    double b = 2.0 * s * P.m * kpad(2 * P.n);                 // GEMM2 B slices
    return std::max(a, b) + 8.0 * P.m + 8.0 * P.n;            // + exponents
}

double split_stageB_bytes_per_item(rt_ctx* c) {
    const Plan& P = c->plan;
    const int s = c->cfg.slices;
    int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
    double a = 2.0 * s * ncmax * kpad(2 * ncmax) + 4.0 * ncmax;  // GEMM3 A slices
    double b = 2.0 * s * P.m * kpad(2 * P.n) + 4.0 * P.m;        // GEMM4 B slices
    return std::max(a, b);
}

void split_alloc_work(rt_ctx* c, int pair_chunk, int item_chunk) {
    SplitState* S = state(c);
    size_t bytes = (size_t)std::max(split_stageA_bytes_per_pair(c) * pair_chunk,
                                    split_stageB_bytes_per_item(c) * item_chunk);
    const Plan& P = c->plan;
    int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
    long long e_pp = 1;
    for (long long v : P.pg_e_pp) e_pp = std::max(e_pp, v);
    size_t rows = std::max({(size_t)e_pp * pair_chunk, (size_t)P.m * pair_chunk,
                            (size_t)ncmax * item_chunk, (size_t)P.m * item_chunk});
    sfree(S, S->a_sl);
    sfree(S, S->a_exp);
    sfree(S, S->b_exp);
    S->a_sl = nullptr;
    S->a_exp = S->b_exp = nullptr;
    S->a_cap = S->a_exp_cap = S->b_exp_cap = 0;
    S->a_sl = (__nv_bfloat16*)salloc(S, bytes);  // A and B slices share the arena in turn
    S->a_cap = bytes;
    S->a_exp = (int*)salloc(S, rows * sizeof(int));
    S->a_exp_cap = rows;
    S->b_exp = (int*)salloc(S, rows * sizeof(int));
    S->b_exp_cap = rows;
}


size_t split_work_bytes(rt_ctx* c) {
    const SplitState* S = c->split;
    return S ? S->a_cap + (S->a_exp_cap + S->b_exp_cap) * sizeof(int) : 0;
}

double split_flop_factor(rt_ctx* c) {
    const int s = c->cfg.slices;
    return s * (s + 1) / 2.0;
}

// Tensor map of an operand stored as s slices [t][rows][Kp]: one box of
// 32 k x box_rows rows x all s slices per load, landing in shared memory as
// s consecutive 64-byte-swizzled tiles.
static CUtensorMap make_map(SplitState* S, const void* base, long long rows, int Kp, int s,
                            int box_rows = SBM, long long slice_rows = 0) {
    CUtensorMap m;
    if (slice_rows <= 0) slice_rows = rows;  // rows between consecutive slices
    cuuint64_t gd[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)s};
    cuuint64_t gs[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)slice_rows * Kp * 2};
    cuuint32_t box[3] = {(cuuint32_t)SBK, (cuuint32_t)box_rows, (cuuint32_t)s};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = S->encode(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), gd, gs,
                           box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(RT_ERR_PROGRAM, "cuTensorMapEncodeTiled failed");
    return m;
}

template <class Epi>
static void run_gemm(rt_ctx* c, const void* a_sl, const int* a_exp, long long M, const void* b_sl,
                     const int* b_exp, long long N, int K, int Kp, Epi epi, int* launches,
                     int ksplit = 1, int kcb = 0, long long b_slice_rows = 0) {
    SplitState* S = state(c);
    if (M <= 0 || N <= 0) return;
    const int s = S->s;
    CUtensorMap ma = make_map(S, a_sl, M, Kp, s);
    CUtensorMap mb = make_map(S, b_sl, N, Kp, s, SBN, b_slice_rows);
    SplitArgs g;
    g.M = M;
    g.N = N;
    g.Kp = Kp;
    g.s = s;
    g.tiles_m = (int)((M + SBM - 1) / SBM);
    g.tiles_n = (int)((N + SBN - 1) / SBN);
    g.ksplit = ksplit;
    g.kcb = ksplit > 1 ? kcb : Kp / SBK;
    if (ksplit > 1) {  // every split non-empty, exact in depth (narrow), all of K covered
        const long long nkb = Kp / SBK;
        if (kcb < 1 || kcb * SBK > KMAX_NARROW || (long long)(ksplit - 1) * kcb >= nkb ||
            (long long)ksplit * kcb < nkb)
            throw Error(RT_ERR_INTERNAL, "inconsistent split-K layout");
    }
    g.row_exp = a_exp;
    g.col_exp = b_exp;
    g.error = S->d_err;
    const bool nocp = test_no_copies();
    const unsigned long long wait_ns = nocp ? 50000000ull : WAIT_NS;
    // CTA pairs (256 rows per pair tile) unless one 128-row tile covers M
    if (ksplit == 1 && M > SBM && S->max_pairs >= 1 && S->use_pairs) {
        CUtensorMap ma2 = make_map(S, a_sl, M, Kp, s, PBM / 2);
        CUtensorMap mb2 = make_map(S, b_sl, N, Kp, s, PBN / 2, b_slice_rows);
        g.tiles_m = (int)((M + PBM - 1) / PBM);
        g.tiles_n = (int)((N + PBN - 1) / PBN);
        const long long strips = std::max<long long>(g.tiles_m, g.tiles_n);
        const int npairs = (int)std::min<long long>(strips, S->max_pairs);
        c->ktimer.begin();
        k_split_gemm_pair<Epi><<<2 * npairs, GEMM_THREADS, pair_smem_bytes(s), c->stream>>>(
            ma2, mb2, g, epi, wait_ns, nocp ? 1 : 0);
        c->ktimer.end(2.0 * (g.tiles_m * (double)PBM) * N * Kp * (s * (s + 1) / 2), 2.0 * M * (double)N * K);
        ++*launches;
        RT_CUDA(cudaGetLastError());
        return;
    }
    const long long ntiles = (long long)g.tiles_m * g.tiles_n * g.ksplit;
    const int grid = (int)std::min<long long>(ntiles, S->num_sms);
    const size_t smem = (size_t)NSTAGE * s * (SBM + SBN) * SBK * 2 + 1024;
    c->ktimer.begin();
    k_split_gemm<128, Epi><<<grid, GEMM_THREADS, smem, c->stream>>>(ma, mb, g, epi, wait_ns, nocp ? 1 : 0);
    // executed tensor FLOPs: s(s+1)/2 digit products over the padded K
    c->ktimer.end(2.0 * M * (double)N * Kp * (s * (s + 1) / 2), 2.0 * M * (double)N * K);
    ++*launches;
    RT_CUDA(cudaGetLastError());
}

std::string split_status_text(int e, bool* unconfirmed) {
    static const char* what[] = {"", "waiting for a free pipeline stage", "waiting for operand tiles",
                                 "waiting for the TMEM accumulators"};
    const int first = e & 0xff;
    std::string t = "split GEMM gave up " + std::string(first >= 1 && first <= 3 ? what[first] : "waiting") +
                    " (status " + std::to_string(e) + ")";
    *unconfirmed = (e & (ERR_DRAIN_UNCONFIRMED | ERR_COPIES_UNCONFIRMED)) != 0;
    if (*unconfirmed)
        t += "; its clean-up could not confirm that all tensor-core work and copies had finished";
    return t;
}

static void check_error(rt_ctx* c) {
    SplitState* S = state(c);
    int e = 0;
    RT_CUDA(cudaMemcpyAsync(&e, S->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    RT_CUDA(cudaStreamSynchronize(c->stream));
    if (e) {
        bool unconfirmed = false;
        const std::string msg = split_status_text(e, &unconfirmed);
        if (unconfirmed) c->unusable = true;
        RT_CUDA(cudaMemset(S->d_err, 0, sizeof(int)));
        throw Error(RT_ERR_PROGRAM, msg);
    }
}

void split_check(rt_ctx* c) { check_error(c); }

__nv_bfloat16* split_a1_slices(rt_ctx* c) { return state(c)->a_sl; }
int* split_a1_exps(rt_ctx* c) { return state(c)->a_exp; }

// GEMM1 of one group on the slices the bucket expansion wrote
void split_gemm1(rt_ctx* c, const G1Group& gg, int npc, const EpiHA& e, int* launches) {
    SplitState* S = state(c);
    const Plan& P = c->plan;
    const int nr = P.blk_size[gg.rblk], nk = P.blk_size[gg.kblk], Kp = kpad(nk);
    const long long M = (long long)nr * npc;
    const ConstSlices& B = S->qap[gg.kblk];
    EpiFF_HA epi{(float2*)e.ha, e.r0, e.m, e.npc, e.plane};
    run_gemm(c, S->a_sl + gg.a_pp * npc, S->a_exp + gg.e_pp * npc, M, B.d, B.exps, 2LL * P.m, nk,
             Kp, epi, launches);
}

// operand slicing of GEMM2/4 (B = float-float K x N) and GEMM3 (A = M3 rows)
void split_prep_gemm24(rt_ctx* c, const double* Bsrc, int K, long long N, cudaStream_t st,
                       int* launches) {
    SplitState* S = state(c);
    launch_slice_cols(S->s, (const float2*)Bsrc, N, K, N, kpad(K), S->b_exp, S->a_sl, st);
    ++*launches;
}

void split_prep_gemm3(rt_ctx* c, const double* m3, int nc, int nij, cudaStream_t st,
                      int* launches) {
    SplitState* S = state(c);
    const int K = 2 * nc;
    launch_slice_rows(S->s, RowsFF{(const float2*)m3, (long long)K}, (long long)nc * nij, K, kpad(K),
                      S->a_sl, S->a_exp, st);
    ++*launches;
}

void split_gemm24(rt_ctx* c, const double* Bsrc, int K, long long N, const EpiRowMajor& e,
                  int* launches) {
    SplitState* S = state(c);
    const int Kp = kpad(K);
    split_prep_gemm24(c, Bsrc, K, N, c->stream, launches);
    EpiFF_RowMajor epi{(float2*)e.c, e.ldc};
    run_gemm(c, S->qah.d, S->qah.exps, S->qah.rows, S->a_sl, S->b_exp, N, K, Kp, epi, launches);
}

// GEMM2 restricted to the blocks of RI = QA^H G QA that the Kramers
// selection reads (internal order: unbarred spinors [0, m/2), barred
// [m/2, m)): all rows against the unbarred columns, the barred rows against
// the barred columns; the unbarred-row x barred-column block is not formed.
// N = m * npc columns ordered (b, pq).
void split_gemm2_kramers(rt_ctx* c, const double* Bsrc, int K, long long N, const EpiRowMajor& e,
                         int* launches) {
    SplitState* S = state(c);
    const int m = c->plan.m, Kh = m / 2, Kp = kpad(K);
    const long long npc = N / m, nh = (long long)Kh * npc;
    split_prep_gemm24(c, Bsrc, K, N, c->stream, launches);
    EpiFF_RowMajor e1{(float2*)e.c, e.ldc};
    run_gemm(c, S->qah.d, S->qah.exps, S->qah.rows, S->a_sl, S->b_exp, nh, K, Kp, e1, launches, 1, 0,
             N);
    EpiFF_RowMajor e2{(float2*)e.c, e.ldc, Kh, m, nh};
    run_gemm(c, S->qahB.d, S->qahB.exps, S->qahB.rows, S->a_sl + (size_t)nh * Kp, S->b_exp + nh, nh,
             K, Kp, e2, launches, 1, 0, N);
}

void split_gemm3(rt_ctx* c, int comp, const double* m3, int nc, int nij, const EpiRK& e,
                 int* launches) {
    SplitState* S = state(c);
    const int K = 2 * nc, Kp = kpad(K);
    const long long M = (long long)nc * nij;
    split_prep_gemm3(c, m3, nc, nij, c->stream, launches);
    const ConstSlices& B = S->qar[comp];
    EpiFF_RK epi{(float2*)e.rk, e.m, e.rowoff, e.plane};
    run_gemm(c, S->a_sl, S->a_exp, M, B.d, B.exps, 2LL * c->plan.m, K, Kp, epi, launches);
}

// Gaunt stage A: RIA = QA^H HA over all blocks and RI2 = QB^H HA over the
// small-component rows of HA (trans1.F:81-97), both from one slicing of HA.
void split_gemm2_breit(rt_ctx* c, const double* Bsrc, int K, long long N, const EpiRowMajor& ria,
                       const EpiRowMajor& ri2, int* launches) {
    SplitState* S = state(c);
    const int Kp = kpad(K);
    split_prep_gemm24(c, Bsrc, K, N, c->stream, launches);
    run_gemm(c, S->qah.d, S->qah.exps, S->qah.rows, S->a_sl, S->b_exp, N, K, Kp,
             EpiFF_RowMajor{(float2*)ria.c, ria.ldc}, launches);
    run_gemm(c, S->qbhS.d, S->qbhS.exps, S->qbhS.rows, S->a_sl, S->b_exp, N, K, Kp,
             EpiFF_RowMajor{(float2*)ri2.c, ri2.ldc}, launches);
}

// GEMM3 of a rectangular expansion: rows (p, ij) of row component `rcomp`
// (nrow functions), K = 2 ncol over the functions of component kcomp, B =
// [[Q_r, Q_i], [-Q_i, Q_r]] of QA (op 0) or QB (op 1).
void split_gemm3_op(rt_ctx* c, int op, int kcomp, const double* m3, int nrow, int ncol, int nij,
                    const EpiRK& e, int* launches) {
    SplitState* S = state(c);
    const int K = 2 * ncol, Kp = kpad(K);
    const long long M = (long long)nrow * nij;
    launch_slice_rows(S->s, RowsFF{(const float2*)m3, (long long)K}, M, K, Kp, S->a_sl, S->a_exp, c->stream);
    ++*launches;
    const ConstSlices& B = op ? S->qbr[kcomp] : S->qar[kcomp];
    EpiFF_RK epi{(float2*)e.rk, e.m, e.rowoff, e.plane};
    run_gemm(c, S->a_sl, S->a_exp, M, B.d, B.exps, 2LL * c->plan.m, K, Kp, epi, launches);
}

// GEMM4 with A = QA^H (op 0) or QB^H (op 1)
void split_gemm4_op(rt_ctx* c, int op, const double* Bsrc, int K, long long N, const EpiRowMajor& e,
                    int* launches) {
    SplitState* S = state(c);
    const int Kp = kpad(K);
    split_prep_gemm24(c, Bsrc, K, N, c->stream, launches);
    const ConstSlices& A = op ? S->qbh : S->qah;
    run_gemm(c, A.d, A.exps, A.rows, S->a_sl, S->b_exp, N, K, Kp, EpiFF_RowMajor{(float2*)e.c, e.ldc},
             launches);
}

// ---------------------------------------------------------------------------
// grouped launches: the same GEMM stage of many transforms in one
// persistent launch over all their tiles (tables built once, launched many
// times; tile width 128 or 64 chosen per group)
// ---------------------------------------------------------------------------
struct GroupProblem {
    const void* a_sl;
    const int* a_exp;
    long long M;
    const void* b_sl;
    const int* b_exp;
    long long N;
    int K, Kp;
    long long b_slice_rows;  // rows between B slices (0: N)
};

struct SplitGroup {
    int kind = 0;  // 0: GEMM1 (EpiFF_HA), 1: GEMM2/4 (EpiFF_RowMajor), 2: GEMM3 (EpiFF_RK)
    int s = 6;
    std::vector<GroupProblem> probs;
    std::vector<EpiFF_HA> e1;
    std::vector<EpiFF_RowMajor> e24;
    std::vector<EpiFF_RK> e3;
    PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    int num_sms = 152;
    // device tables per tile width (index 0: 128, 1: 64)
    void* d_args[2] = {nullptr, nullptr};
    void* d_maps[2] = {nullptr, nullptr};
    void* d_start[2] = {nullptr, nullptr};
    void* d_epi = nullptr;
    long long ntiles[2] = {0, 0};
    double flops_exec = 0.0, flops_alg = 0.0;
};

SplitGroup* split_group_new(int kind) {
    SplitGroup* g = new SplitGroup();
    g->kind = kind;
    return g;
}

void split_group_add_gemm1(SplitGroup* G, rt_ctx* c, const G1Group& gg, int npc, const EpiHA& e) {
    SplitState* S = state(c);
    const Plan& P = c->plan;
    const int nr = P.blk_size[gg.rblk], nk = P.blk_size[gg.kblk];
    const ConstSlices& B = S->qap[gg.kblk];
    G->probs.push_back({S->a_sl + gg.a_pp * npc, S->a_exp + gg.e_pp * npc, (long long)nr * npc, B.d,
                        B.exps, 2LL * P.m, nk, kpad(nk), 0});
    G->e1.push_back(EpiFF_HA{(float2*)e.ha, e.r0, e.m, e.npc, e.plane});
    G->s = S->s;
}

void split_group_add_gemm24(SplitGroup* G, rt_ctx* c, int K, long long N, const EpiRowMajor& e) {
    SplitState* S = state(c);
    G->probs.push_back({S->qah.d, S->qah.exps, (long long)S->qah.rows, S->a_sl, S->b_exp, N, K,
                        kpad(K), 0});
    G->e24.push_back(EpiFF_RowMajor{(float2*)e.c, e.ldc});
    G->s = S->s;
}

// the two launches of split_gemm2_kramers as two problems of a group
void split_group_add_gemm2_kramers(SplitGroup* G, rt_ctx* c, int K, long long N, const EpiRowMajor& e) {
    SplitState* S = state(c);
    const int m = c->plan.m, Kh = m / 2, Kp = kpad(K);
    const long long nh = (long long)Kh * (N / m);
    G->probs.push_back({S->qah.d, S->qah.exps, (long long)S->qah.rows, S->a_sl, S->b_exp, nh, K, Kp, N});
    G->e24.push_back(EpiFF_RowMajor{(float2*)e.c, e.ldc});
    G->probs.push_back({S->qahB.d, S->qahB.exps, (long long)S->qahB.rows, S->a_sl + (size_t)nh * Kp,
                        S->b_exp + nh, nh, K, Kp, N});
    G->e24.push_back(EpiFF_RowMajor{(float2*)e.c, e.ldc, Kh, m, nh});
    G->s = S->s;
}

void split_group_add_gemm3(SplitGroup* G, rt_ctx* c, int comp, int nc, int nij, const EpiRK& e) {
    SplitState* S = state(c);
    const ConstSlices& B = S->qar[comp];
    G->probs.push_back({S->a_sl, S->a_exp, (long long)nc * nij, B.d, B.exps, 2LL * c->plan.m, 2 * nc,
                        kpad(2 * nc), 0});
    G->e3.push_back(EpiFF_RK{(float2*)e.rk, e.m, e.rowoff, e.plane});
    G->s = S->s;
}

template <class Epi>
static void set_group_smem(const cudaDeviceProp& prop) {
    set_smem_limit(k_split_gemm_grouped<128, Epi>, (size_t)NSTAGE * MAX_SLICES * (SBM + 128) * SBK * 2 + 1024, prop);
    set_smem_limit(k_split_gemm_grouped<64, Epi>, (size_t)NSTAGE * MAX_SLICES * (SBM + 64) * SBK * 2 + 1024, prop);
}

// Encode the tensor maps of both tile widths and upload the tables.
void split_group_build(SplitGroup* G, rt_ctx* c0) {
    SplitState* S = state(c0);
    G->encode = S->encode;
    G->num_sms = S->num_sms;
    static bool smem_set[64] = {};
    int dev = 0;
    RT_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && !smem_set[dev]) {
        cudaDeviceProp prop;
        RT_CUDA(cudaGetDeviceProperties(&prop, dev));
        set_group_smem<EpiFF_HA>(prop);
        set_group_smem<EpiFF_RowMajor>(prop);
        set_group_smem<EpiFF_RK>(prop);
        smem_set[dev] = true;
    }
    const int np = (int)G->probs.size();
    if (np == 0) return;
    SplitState tmp;
    tmp.encode = G->encode;
    for (int v = 0; v < 2; ++v) {
        const int bn = v == 0 ? 128 : 64;
        std::vector<SplitArgs> args(np);
        std::vector<CUtensorMap> maps(2 * (size_t)np);
        std::vector<long long> start(np + 1, 0);
        for (int p = 0; p < np; ++p) {
            const GroupProblem& q = G->probs[p];
            SplitArgs& a = args[p];
            a.M = q.M;
            a.N = q.N;
            a.Kp = q.Kp;
            a.s = G->s;
            a.tiles_m = (int)((q.M + SBM - 1) / SBM);
            a.tiles_n = (int)((q.N + bn - 1) / bn);
            a.ksplit = 1;
            a.kcb = q.Kp / SBK;
            a.row_exp = q.a_exp;
            a.col_exp = q.b_exp;
            a.error = nullptr;
            maps[2 * p] = make_map(&tmp, q.a_sl, q.M, q.Kp, G->s, SBM);
            maps[2 * p + 1] = make_map(&tmp, q.b_sl, q.N, q.Kp, G->s, bn, q.b_slice_rows);
            start[p + 1] = start[p] + (q.M > 0 && q.N > 0 ? (long long)a.tiles_m * a.tiles_n : 0);
            if (v == 0) {
                G->flops_exec += 2.0 * q.M * (double)q.N * q.Kp * (G->s * (G->s + 1) / 2);
                G->flops_alg += 2.0 * q.M * (double)q.N * q.K;
            }
        }
        G->ntiles[v] = start[np];
        RT_CUDA(cudaMalloc(&G->d_args[v], args.size() * sizeof(SplitArgs)));
        RT_CUDA(cudaMalloc(&G->d_maps[v], maps.size() * sizeof(CUtensorMap)));
        RT_CUDA(cudaMalloc(&G->d_start[v], start.size() * sizeof(long long)));
        RT_CUDA(cudaMemcpy(G->d_args[v], args.data(), args.size() * sizeof(SplitArgs), cudaMemcpyHostToDevice));
        RT_CUDA(cudaMemcpy(G->d_maps[v], maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
        RT_CUDA(cudaMemcpy(G->d_start[v], start.data(), start.size() * sizeof(long long), cudaMemcpyHostToDevice));
    }
    size_t eb = 0;
    const void* src = nullptr;
    if (G->kind == 0) { eb = G->e1.size() * sizeof(EpiFF_HA); src = G->e1.data(); }
    if (G->kind == 1) { eb = G->e24.size() * sizeof(EpiFF_RowMajor); src = G->e24.data(); }
    if (G->kind == 2) { eb = G->e3.size() * sizeof(EpiFF_RK); src = G->e3.data(); }
    RT_CUDA(cudaMalloc(&G->d_epi, eb));
    RT_CUDA(cudaMemcpy(G->d_epi, src, eb, cudaMemcpyHostToDevice));
}

template <int BN, class Epi>
static void group_launch(SplitGroup* G, int v, cudaStream_t st, int* err) {
    GroupTable<Epi> tab;
    tab.g = (const SplitArgs*)G->d_args[v];
    tab.maps = (const CUtensorMap*)G->d_maps[v];
    tab.e = (const Epi*)G->d_epi;
    tab.start = (const long long*)G->d_start[v];
    tab.nprob = (int)G->probs.size();
    const int grid = (int)std::min<long long>(G->ntiles[v], G->num_sms);
    const size_t smem = (size_t)NSTAGE * G->s * (SBM + BN) * SBK * 2 + 1024;
    k_split_gemm_grouped<BN, Epi><<<grid, GEMM_THREADS, smem, st>>>(tab, G->s, err);
}

// One persistent launch over all tiles of the group, tile width bn (128/64).
void split_group_launch(SplitGroup* G, int bn, cudaStream_t st, int* err) {
    if (G->probs.empty()) return;
    const int v = bn == 64 ? 1 : 0;
    if (G->ntiles[v] == 0) return;
    if (G->kind == 0) (v ? group_launch<64, EpiFF_HA> : group_launch<128, EpiFF_HA>)(G, v, st, err);
    if (G->kind == 1) (v ? group_launch<64, EpiFF_RowMajor> : group_launch<128, EpiFF_RowMajor>)(G, v, st, err);
    if (G->kind == 2) (v ? group_launch<64, EpiFF_RK> : group_launch<128, EpiFF_RK>)(G, v, st, err);
    RT_CUDA(cudaGetLastError());
}

int split_group_size(const SplitGroup* G) { return (int)G->probs.size(); }

std::string split_group_shape(const SplitGroup* g) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "kind%d:s%d:p%zu:t%lld:t%lld:f%d", g->kind, g->s, g->probs.size(),
                  g->ntiles[0], g->ntiles[1],
                  g->flops_exec > 0 ? (int)std::lround(std::log2(g->flops_exec)) : 0);
    return buf;
}
double split_group_flops(const SplitGroup* G, bool executed) {
    return executed ? G->flops_exec : G->flops_alg;
}

void split_group_free(SplitGroup* G) {
    if (!G) return;
    for (int v = 0; v < 2; ++v) {
        cudaFree(G->d_args[v]);
        cudaFree(G->d_maps[v]);
        cudaFree(G->d_start[v]);
    }
    cudaFree(G->d_epi);
    delete G;
}

// ---------------------------------------------------------------------------
// long rows (operands of the adjoint contraction, K up to ~10^8): exponents
// by a block-parallel maximum, then the digits elementwise
// ---------------------------------------------------------------------------
constexpr int LONG_BLOCK = SPLIT_LONG_BLOCK;  // K per split of the contraction = per exponent

// exps[kb * rows + row] = exponent of row's K block kb (LONG_BLOCK deep)
__global__ void __launch_bounds__(256) k_rowexp_long(const float2* __restrict__ src, long long ld,
                                                     int rows, long long K, int* __restrict__ exps) {
    __shared__ int wmax[8];
    const int row = blockIdx.y, kb = blockIdx.x;
    const long long k0 = (long long)kb * LONG_BLOCK;
    const long long k1 = min(K, k0 + LONG_BLOCK);
    int S = -2000;
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x)
        S = max(S, scale_exp_f32(src[(long long)row * ld + k].x, slicing_wide(LONG_BLOCK)));
    for (int o = 16; o; o >>= 1) S = max(S, __shfl_xor_sync(0xffffffffu, S, o));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = S;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; ++w) S = max(S, wmax[w]);
        exps[(long long)kb * rows + row] = S;
    }
}

// digits of row's K block blockIdx.x (LONG_BLOCK / 4 threads x 4 consecutive k)
template <int NS>
__global__ void __launch_bounds__(256) k_slice_rows_long(const float2* __restrict__ src, long long ld,
                                                         int rows, long long K, long long Kp,
                                                         const int* __restrict__ exps,
                                                         __nv_bfloat16* __restrict__ out) {
    const int row = blockIdx.y;
    const long long k0 = (long long)blockIdx.x * LONG_BLOCK + threadIdx.x * 4;
    if (k0 >= Kp) return;
    const int S = exps[(long long)blockIdx.x * rows + row];
    const float sc = pow2f_safe(-S);
    __nv_bfloat16 d[4][NS];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float2 v = make_float2(0.f, 0.f);
        if (k0 + j < K && S > -1000) v = src[(long long)row * ld + k0 + j];
        ff_digits<NS>(v.x * sc, v.y * sc, d[j]);
    }
#pragma unroll
    for (int t = 0; t < NS; ++t) {
        uint2 w = make_uint2(pack_bf16x2(d[0][t], d[1][t]), pack_bf16x2(d[2][t], d[3][t]));
        *reinterpret_cast<uint2*>(out + ((long long)t * rows + row) * Kp + k0) = w;
    }
}

// slices [s][rows][Kp] and exponents [Kp/LONG_BLOCK][rows] of long rows
static void slice_long_rows(int s, const float2* src, long long ld, int rows, long long K,
                            long long Kp, int* exps, __nv_bfloat16* out, cudaStream_t st) {
    if (rows > 65535) throw Error(RT_ERR_DIM, "long-row slicing: more than 65535 rows");
    dim3 g((unsigned)((Kp + LONG_BLOCK - 1) / LONG_BLOCK), (unsigned)rows);
    k_rowexp_long<<<g, 256, 0, st>>>(src, ld, rows, K, exps);
    constexpr int T = LONG_BLOCK / 4;  // one thread per 4 k of the block
    static_assert(LONG_BLOCK % 128 == 0 && T <= 256, "long-row block of whole warps");
    switch (s) {
        case 2: k_slice_rows_long<2><<<g, T, 0, st>>>(src, ld, rows, K, Kp, exps, out); break;
        case 3: k_slice_rows_long<3><<<g, T, 0, st>>>(src, ld, rows, K, Kp, exps, out); break;
        case 4: k_slice_rows_long<4><<<g, T, 0, st>>>(src, ld, rows, K, Kp, exps, out); break;
        case 5: k_slice_rows_long<5><<<g, T, 0, st>>>(src, ld, rows, K, Kp, exps, out); break;
        default: k_slice_rows_long<6><<<g, T, 0, st>>>(src, ld, rows, K, Kp, exps, out); break;
    }
}

// Adjoint X GEMM of one component: rows (p, ij, plane) of the float-float
// M3 times [QAr | QAi] of the component, into X[a][ij][plane][ri][k].
void split_adj_x(rt_ctx* c, int comp, const double* m3, int nc, int nij, double* x,
                 __nv_bfloat16* sl, int* ex, int* launches) {
    SplitState* S = state(c);
    const int m = c->plan.m, Kp = kpad(nc);
    const long long M = 2LL * nc * nij;
    launch_slice_rows(S->s, RowsFF{(const float2*)m3, (long long)nc}, M, nc, Kp, sl, ex, c->stream);
    ++*launches;
    const ConstSlices& B = S->qc[comp];
    EpiFF_RowMajor epi{(float2*)(x + (size_t)c->plan.comp_off[comp] * nij * 4 * m), 2LL * m};
    run_gemm(c, sl, ex, M, B.d, B.exps, 2LL * m, nc, Kp, epi, launches);
}

long long split_adj_kpad(long long K) { return (K + SBK - 1) / SBK * SBK; }

// Adjoint contraction part[ks][a][col] = sum over split ks of X(a,k) Ghat(k,col)
// with Ghat given transposed (rows col, length Kx); every LONG_BLOCK-deep split
// has its own row and column scales (a_ex: [ks][rows], b_ex: [ks][2m]).
// Returns the split count.
int split_adj_contract(rt_ctx* c, const double* x, int rows, long long Kx, const double* ghat_t,
                       __nv_bfloat16* a_sl, int* a_ex, __nv_bfloat16* b_sl, int* b_ex, double* part,
                       int* launches) {
    SplitState* S = state(c);
    const int m2 = 2 * c->plan.m;
    const long long Kp = split_adj_kpad(Kx);
    if (Kp > (1LL << 30)) throw Error(RT_ERR_DIM, "adjoint contraction: K above 2^30");
    slice_long_rows(S->s, (const float2*)x, Kx, rows, Kx, Kp, a_ex, a_sl, c->stream);
    slice_long_rows(S->s, (const float2*)ghat_t, Kx, m2, Kx, Kp, b_ex, b_sl, c->stream);
    *launches += 4;
    RT_CUDA(cudaGetLastError());
    // one split per exponent block; LONG_BLOCK <= 819 keeps the narrow FP32 sums exact
    const int kcb = LONG_BLOCK / SBK;
    const int nkb = (int)(Kp / SBK);
    const int ksplit = (nkb + kcb - 1) / kcb;
    run_gemm(c, a_sl, a_ex, rows, b_sl, b_ex, m2, (int)Kx, (int)Kp,
             EpiFF_RowMajor{(float2*)part, (long long)m2}, launches, ksplit, kcb);
    return ksplit;
}

void split_release(rt_ctx* c) {
    if (!c->split) return;
    for (void* p : c->split->allocs) cudaFree(p);
    delete c->split;
    c->split = nullptr;
}

}  // namespace rt

extern "C" int rt_split_dgemm(int M, int N, int K, const double* A, const double* B, double* C,
                              int slices, int mode) {
    using namespace rt;
    if (K > 1024) return RT_ERR_DIM;  // the engine's tested depth; exact up to 1365
    if (M < 1 || N < 1 || K < 1 || !A || !B || !C || slices < 2 ||
        slices > MAX_SLICES || mode < 0 || mode > 2)
        return RT_ERR_USER;
    rt_ctx ctx;
    int rc = RT_OK;
    std::vector<void*> tmp;
    auto dal = [&](size_t bytes) {
        void* p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) throw Error(RT_ERR_DIM, "allocation failed");
        tmp.push_back(p);
        return p;
    };
    try {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw Error(RT_ERR_PROGRAM, "no CUDA device");
        RT_CUDA(cudaGetDevice(&ctx.device));
        RT_CUDA(cudaStreamCreateWithFlags(&ctx.stream, cudaStreamNonBlocking));
        ctx.ktimer.reset(ctx.stream);
        ctx.cfg.slices = slices;
        SplitState* S = state(&ctx);
        const int Kp = kpad(K);
        int launches = 0;
        __nv_bfloat16 *da, *db;
        int *ea, *eb;
        if (mode == 0) {
            std::vector<uint16_t> sl;
            std::vector<int> ex;
            std::vector<double> av(A, A + (size_t)M * K);
            host_slice_rows(av, M, K, Kp, slices, sl, ex);
            da = (__nv_bfloat16*)dal(sl.size() * 2);
            ea = (int*)dal(ex.size() * 4);
            RT_CUDA(cudaMemcpy(da, sl.data(), sl.size() * 2, cudaMemcpyHostToDevice));
            RT_CUDA(cudaMemcpy(ea, ex.data(), ex.size() * 4, cudaMemcpyHostToDevice));
            host_slice_cols(B, K, N, N, Kp, slices, sl, ex);
            db = (__nv_bfloat16*)dal(sl.size() * 2);
            eb = (int*)dal(ex.size() * 4);
            RT_CUDA(cudaMemcpy(db, sl.data(), sl.size() * 2, cudaMemcpyHostToDevice));
            RT_CUDA(cudaMemcpy(eb, ex.data(), ex.size() * 4, cudaMemcpyHostToDevice));
        } else {
            da = (__nv_bfloat16*)dal((size_t)2 * slices * M * Kp);
            ea = (int*)dal((size_t)4 * M);
            db = (__nv_bfloat16*)dal((size_t)2 * slices * N * Kp);
            eb = (int*)dal((size_t)4 * N);
            std::vector<float2> bf((size_t)K * N);
            for (size_t i = 0; i < bf.size(); ++i) {
                float h = (float)B[i];
                bf[i] = make_float2(h, (float)(B[i] - (double)h));
            }
            float2* dbf = (float2*)dal(bf.size() * 8);
            RT_CUDA(cudaMemcpy(dbf, bf.data(), bf.size() * 8, cudaMemcpyHostToDevice));
            launch_slice_cols(slices, dbf, N, K, N, Kp, eb, db, ctx.stream);
            if (mode == 1) {
                std::vector<float2> af((size_t)M * K);
                for (size_t i = 0; i < af.size(); ++i) {
                    float h = (float)A[i];
                    af[i] = make_float2(h, (float)(A[i] - (double)h));
                }
                float2* daf = (float2*)dal(af.size() * 8);
                RT_CUDA(cudaMemcpy(daf, af.data(), af.size() * 8, cudaMemcpyHostToDevice));
                launch_slice_rows(slices, RowsFF{daf, K}, M, K, Kp, da, ea, ctx.stream);
            } else {
                double* dad = (double*)dal((size_t)M * K * 8);
                RT_CUDA(cudaMemcpy(dad, A, (size_t)M * K * 8, cudaMemcpyHostToDevice));
                RowsF64Batched src{dad, (long long)M, 0, M, K};
                launch_slice_rows(slices, src, M, K, Kp, da, ea, ctx.stream);
            }
            RT_CUDA(cudaGetLastError());
        }
        float2* dc = (float2*)dal((size_t)M * N * 8);
        RT_CUDA(cudaMemsetAsync(dc, 0, (size_t)M * N * 8, ctx.stream));
        run_gemm(&ctx, da, ea, M, db, eb, N, K, Kp, EpiFF_RowMajor{dc, N}, &launches);
        check_error(&ctx);
        std::vector<float2> hc((size_t)M * N);
        RT_CUDA(cudaMemcpy(hc.data(), dc, hc.size() * 8, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < hc.size(); ++i) C[i] = (double)hc[i].x + (double)hc[i].y;
    } catch (const Error& e) {
        rc = e.code;
    }
    for (void* p : tmp) cudaFree(p);
    split_release(&ctx);
    if (ctx.stream) cudaStreamDestroy(ctx.stream);
    return rc;
}

// ---------------------------------------------------------------------------
// rt_split_dgemm_noalloc: the same product on device-resident FP64 matrices
// with every scratch buffer carved from one fixed device array.
// ---------------------------------------------------------------------------
namespace rt {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)48 << 20;
constexpr int NOALLOC_MAX_DEVICES = 64;

// error flag, row/column exponents, A and B slices, float-float copy of B
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocDevice {
    unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
    int num_sms = 0;
    bool unusable = false;  // an aborted GEMM could not confirm its clean-up
};
static NoallocDevice g_noalloc_dev[NOALLOC_MAX_DEVICES];
static PFN_cuTensorMapEncodeTiled_v12000 g_noalloc_encode = nullptr;
static std::mutex g_noalloc_mutex;

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

static size_t noalloc_bytes(long long M, long long N, int K, int s) {
    const long long Kp = kpad(K);
    return 256 + align256(4 * (size_t)M) + align256(4 * (size_t)N) +
           align256((size_t)2 * s * M * Kp) + align256((size_t)2 * s * N * Kp) +
           align256((size_t)8 * K * N);
}

// FP64 -> float-float with the leading part rounded to nearest (the same
// split the host applies before device slicing)
__global__ void k_ff_round(const double* __restrict__ x, long long n, float2* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = x[i];
        const float h = __double2float_rn(v);
        out[i] = make_float2(h, __double2float_rn(v - (double)h));
    }
}

// Is [p, p + bytes) memory the current device `dev` can read and write?
// Device memory of dev (the whole range inside one allocation), managed
// memory, or page-locked host memory mapped at the same address; not
// pageable host memory, and not memory of another device.
static bool device_range_ok(const void* p, size_t bytes, int dev) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    if (a.type == cudaMemoryTypeHost) return a.devicePointer == p;
    if (a.type != cudaMemoryTypeDevice || a.device != dev) return false;
    static PFN_cuMemGetAddressRange_v3020 range = nullptr;
    if (!range) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &fn, 3020, cudaEnableDefault, &q) !=
                cudaSuccess ||
            !fn || q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return true;  // the type check above stands alone
        }
        range = (PFN_cuMemGetAddressRange_v3020)fn;
    }
    CUdeviceptr base = 0;
    size_t size = 0;
    if (range(&base, &size, (CUdeviceptr)(uintptr_t)p) != CUDA_SUCCESS) return false;
    return (uintptr_t)p + bytes <= (uintptr_t)base + size;
}

// Per-device set-up, with that device current: the device address of the
// scratch array, the SM count and the GEMM's shared-memory limit.
static const NoallocDevice& noalloc_setup(int dev) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoallocDevice& d = g_noalloc_dev[dev];
    if (d.scratch) return d;
    if (!g_noalloc_encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        RT_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                 cudaEnableDefault, &q));
        if (!fn || q != cudaDriverEntryPointSuccess)
            throw Error(RT_ERR_PROGRAM, "cuTensorMapEncodeTiled unavailable");
        g_noalloc_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    cudaDeviceProp prop;
    RT_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (prop.major * 10 + prop.minor != 103)
        throw Error(RT_ERR_PROGRAM, "rt_split_dgemm_noalloc needs an sm_103 device");
    set_smem_limit(k_split_gemm<128, EpiF64_RowMajor>,
                   (size_t)NSTAGE * MAX_SLICES * (SBM + SBN) * SBK * 2 + 1024, prop);
    void* p = nullptr;
    RT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    d.num_sms = prop.multiProcessorCount;
    d.scratch = (unsigned char*)p;
    return d;
}

}  // namespace rt

extern "C" int rt_split_dgemm_noalloc(int M, int N, int K, const double* A, const double* B,
                                      double* C, int slices, void* stream) {
    using namespace rt;
    if (M < 1 || N < 1 || K < 1 || !A || !B || !C || slices < 2 || slices > MAX_SLICES) {
        set_thread_error("rt_split_dgemm_noalloc: M, N, K >= 1, non-null A, B, C and 2 <= slices <= 6 required");
        return RT_ERR_USER;
    }
    if (K > 1024) {
        set_thread_error("rt_split_dgemm_noalloc: K > 1024 (the depth the engine is tested to)");
        return RT_ERR_DIM;
    }
    const size_t need = noalloc_bytes(M, N, K, slices);
    if (need > NOALLOC_SCRATCH_BYTES) {
        set_thread_error("rt_split_dgemm_noalloc: needs " + std::to_string(need) +
                         " bytes of scratch, more than the fixed " +
                         std::to_string(NOALLOC_SCRATCH_BYTES) + " bytes");
        return RT_ERR_DIM;
    }
    try {
        int dev = 0;
        RT_CUDA(cudaGetDevice(&dev));
        if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) throw Error(RT_ERR_DIM, "device ordinal above 63");
        const NoallocDevice& D = noalloc_setup(dev);
        if (D.unusable)
            throw Error(RT_ERR_PROGRAM, "an earlier call on this device was aborted without a confirmed clean-up");
        if (!device_range_ok(A, 8 * (size_t)M * K, dev) || !device_range_ok(B, 8 * (size_t)K * N, dev) ||
            !device_range_ok(C, 8 * (size_t)M * N, dev))
            throw Error(RT_ERR_USER, "A, B and C must be device memory of the current device (or managed, "
                                     "or mapped page-locked host memory) covering M*K, K*N and M*N doubles");
        cudaStream_t st = (cudaStream_t)stream;
        const int s = slices, Kp = kpad(K);
        unsigned char* w = D.scratch;
        int* err = (int*)w;
        w += 256;
        int* ea = (int*)w;
        w += align256(4 * (size_t)M);
        int* eb = (int*)w;
        w += align256(4 * (size_t)N);
        __nv_bfloat16* da = (__nv_bfloat16*)w;
        w += align256((size_t)2 * s * M * Kp);
        __nv_bfloat16* db = (__nv_bfloat16*)w;
        w += align256((size_t)2 * s * N * Kp);
        float2* bff = (float2*)w;
        // the slicing kernels write every element they are asked for; only
        // the error flag has to start at zero
        RT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
        const long long nb = (long long)K * N;
        k_ff_round<<<(unsigned)std::min<long long>((nb + 255) / 256, 152LL * 16), 256, 0, st>>>(B, nb, bff);
        launch_slice_cols(s, bff, N, K, N, Kp, eb, db, st);
        launch_slice_rows(s, RowsF64Batched{A, (long long)M, 0, M, K}, M, K, Kp, da, ea, st);
        RT_CUDA(cudaGetLastError());
        SplitState S;
        S.encode = g_noalloc_encode;
        CUtensorMap ma = make_map(&S, da, M, Kp, s);
        CUtensorMap mb = make_map(&S, db, N, Kp, s);
        SplitArgs g;
        g.M = M;
        g.N = N;
        g.Kp = Kp;
        g.s = s;
        g.tiles_m = (M + SBM - 1) / SBM;
        g.tiles_n = (N + SBN - 1) / SBN;
        g.ksplit = 1;
        g.kcb = Kp / SBK;
        g.row_exp = ea;
        g.col_exp = eb;
        g.error = err;
        const int grid = std::min(g.tiles_m * g.tiles_n, D.num_sms);
        const size_t smem = (size_t)NSTAGE * s * (SBM + SBN) * SBK * 2 + 1024;
        k_split_gemm<128, EpiF64_RowMajor><<<grid, GEMM_THREADS, smem, st>>>(ma, mb, g, EpiF64_RowMajor{C, N},
                                                                           WAIT_NS, 0);
        RT_CUDA(cudaGetLastError());
        int e = 0;
        RT_CUDA(cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        RT_CUDA(cudaStreamSynchronize(st));
        if (e) {
            bool unconfirmed = false;
            const std::string msg = split_status_text(e, &unconfirmed);
            if (unconfirmed) g_noalloc_dev[dev].unusable = true;
            throw Error(RT_ERR_PROGRAM, msg);
        }
    } catch (const Error& e) {
        set_thread_error("rt_split_dgemm_noalloc: " + e.msg);
        return e.code;
    }
    return RT_OK;
}
