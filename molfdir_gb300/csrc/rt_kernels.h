// rt_kernels.h -- launchers and epilogue functors shared by the transform
// paths.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace rt {

enum : unsigned int {
    ST_BAD_LABEL = 1u,   // a label outside 1..NSC or a non-canonical pq pair
    ST_BAD_BLOCK = 2u,   // an integral outside the (LL|LL),(SS|LL),(SS|SS) / irrep block structure
};

// Index tables of the record bucketing (device pointers).
struct ScatterTabs {
    int n, mfil, nblk;
    const unsigned char* pq_read;  // [n(n+1)/2] rotran transforms this pq bucket (makind.F:70-90)
    const int* pair_of_orig;       // [n(n+1)/2] -> pair order or -1
    const int* pair_group;         // [P] pair group
    const int* pg_start;           // [npg]
    const int* pg_size;            // [npg]
    const int* ao_block;           // [n] AO block
    const int* ao_pos;             // [n] position inside its block
    const int* blk_size;           // [nblk]
    const int* g1_of;              // [npg*nblk] GEMM1 group of (pair group, r block) or -1
    const int* g1_kblk;            // [ng1] partner block of the group
    const int* jb_base;            // [npg*nblk] first expansion job of (pair group, r block)
    const int* jb_band;            // [npg*nblk] rows per band of those jobs
    const long long* pg_bbase;     // [npg] first bucket of the pair group
    const int* pg_njobs;           // [npg] expansion jobs per pair
    int breit = 0;                 // Gaunt integrals: file 4 only, sign turned (gettw.F:51-55)
    int half = 0;                  // rotran's half buckets: LABEL1 pair only (sort1.F:78-142)
};

// One MDCINT record of the current item chunk.
struct EmitRec {
    int ijl;   // item inside the chunk
    int cls;   // 0..3 = MDCINT classes 1..4
    int ikr, jkr;
    int rank;  // record number inside its class stream
};

// The four class streams of the MDCINT record file (device pointers).
struct OutStreams {
    int* cnt[4];        // elements per record
    long long* off[4];  // first element of each record
    int* idx[4];        // (INDK, INDL) pairs
    double* val[4];     // (re, im) pairs
    long long* total;   // [4] running element totals
};

// One band of rows of one GEMM1 group, expanded from the pq buckets.
struct ExpandJob {
    int rblk;         // AO block of r
    int r_lo, r_hi;   // band of r positions inside the block
    int nr;           // rows of the block (the group's r extent)
    int nk;           // columns (size of the partner block)
    int kp;           // padded K of the slices
    long long out_pp;   // offset of the group's operand in the output buffer, per pair
    long long exp_pp;   // offset of the group's row exponents, per pair
};

// GEMM1 (batched over r): row = pq_local, col = plane*m + b
//   -> HA[plane][r_sorted][b][pq_local]
struct EpiHA {
    double* ha;
    int r0, m, npc;
    long long plane;  // n*m*npc
    __device__ __forceinline__ void operator()(int bz, int row, int col, double v) const {
        int pl = col >= m;
        int b = col - pl * m;
        ha[pl * plane + ((long long)(r0 + bz) * m + b) * npc + row] = v;
    }
};

// plain row-major C with leading dimension ldc (batch stride sc)
struct EpiRowMajor {
    double* c;
    long long ldc, sc;
    __device__ __forceinline__ void operator()(int bz, int row, int col, double v) const {
        c[bz * sc + (long long)row * ldc + col] = v;
    }
};

// GEMM3: row = p_local*nij + ijl, col = plane*m + k
//   -> RK[plane][c0 + p][ijl][k] = plane*PS + (c0*nij + row)*m + k
struct EpiRK {
    double* rk;
    int m;
    long long rowoff;  // c0*nij
    long long plane;   // n*nij*m
    __device__ __forceinline__ void operator()(int, int row, int col, double v) const {
        int pl = col >= m;
        int k = col - pl * m;
        rk[pl * plane + (rowoff + row) * m + k] = v;
    }
};

// raises the library's dimension error (defined in rt_api.cu)
[[noreturn]] void throw_dim(const char* what);

template <class Epi>
void gemm_f64(cudaStream_t st, const double* A, long long lda, long long sA, const double* B,
              long long ldb, long long sB, int M, int N, int K, int batch, Epi epi);

// Buckets in two levels: by pq (count, off[P+1], bval/brs, up to two
// entries per integral), then by (pq, expansion job) (jstart/jcount[nb],
// jval/jrs, up to four entries per integral: element and mirror).
void launch_bucket(cudaStream_t st, const double* rint, const int* l2, const int* l1, long long nint,
                   const long long* rec_off, const int2* rec_meta, int nrec, const ScatterTabs& tb,
                   int P, int* count, long long* off, double* bval, int* brs, long long nb,
                   long long* jstart, int* jcount, double* jval, int* jrs, unsigned int* status);
// expansion of one pair chunk: bucket of (pair pql, job j) = bbase + pql * njobs + j
// Raise a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device; never lowered, so kernels recorded earlier with larger
// sizes (CUDA graph nodes of a batch) stay launchable whatever the order of
// later launches.
void raise_dyn_smem(const void* kernel, size_t bytes);
void launch_expand_rows(cudaStream_t st, int nslices, const double* bval, const int* brs,
                        const long long* jstart, const int* jcount, const ExpandJob* jobs, int njobs,
                        long long bbase, int npc, size_t smem, double* out_f64,
                        __nv_bfloat16* out_sl, int* out_exp);
void launch_tr_select(cudaStream_t st, bool ff, const double* ri, int m, int npc, int pq0, int P,
                      const int4* items, const float* item_sign, int nitems,
                      const double* pair_vmx, const float* pair_thr, double thrgen, double* hp,
                      unsigned long long* kept);
// M3 rows p (nrow) against columns q (ncol) of the half-transformed values;
// two: x2 (MATMUL7); ff: float-float values; diag2: x2 on p = q (rotran's
// half buckets, whose MATMUL3 adds the diagonal pair twice)
void launch_expand(cudaStream_t st, const double* hp, int P, int nitems, int it0, int nij,
                   const int* pidx, int nrow, int ncol, double* m3, bool two = false, bool ff = false,
                   bool diag2 = false);
// One Gaunt item: the stored pair (x, y) = (J', I') of UNIQUE(I, J) (internal
// 0-based spinors), their partners, s = -sign(ITRMO(x) ITRMO(y)), and
// TRANS2's conjugation and sign for the item.
struct BreitItem {
    int x, y, xb, yb;
    float s;
    int conj, neg;
};
void launch_trb_select(cudaStream_t st, bool ff, const double* ria, const double* ri2, int m, int npc,
                       int pq0, int P, const BreitItem* items, int nitems, double* hp,
                       unsigned long long* kept);
void launch_emit(cudaStream_t st, bool ff, const double* rlr, int m, int nij, int K,
                 const EmitRec* rec, int nrec, const int* kra, const int* krb, const int* itrmo,
                 double throut, const OutStreams& os);
// RL of the items it0 .. it0+nij-1 into rl_all[item][K][L] as FP64 (re, im):
// MSUMTIM with ISG = isg, plus (Gaunt, else null) the streams rlr_b, rlr_c
void launch_rl_store(cudaStream_t st, bool ff, const double* rlr, const double* rlr_b, const double* rlr_c,
                     int m, int nij, int it0, const int* itrmo, double isg, double* rl_all);
// Records from rotran's two halves: each element is OUTPP1's part of the
// record's own item plus OUTPP2's part of the item that PPSYM adds into it,
// each kept when above THROUT; item_of[b][i][j] is the item of Kramers pair
// indices (i, j), J barred (b = 1) or not (b = 0)
void launch_emit_halves(cudaStream_t st, const double* rl_all, int m, int K, int it0, const EmitRec* rec,
                        int nrec, const int* item_of, const int* kra, const int* krb, double throut,
                        const OutStreams& os);

// ---- adjoint (dE/dC) ----
// Gamma <- (Gamma + Gamma^T) / 2 with Gamma seen as an m^2 x m^2 complex
// matrix over (first pair, second pair): the pair-exchange symmetrisation.
void launch_gamma_sym(cudaStream_t st, double* gamma, int m);
// out(i,j,k,l) = in(u[i],u[j],u[k],u[l]) (complex, Fortran order)
void launch_gamma_permute(cudaStream_t st, const double* in, const int* u, int m, double* out);
// Contraction operand of one item chunk, real-ified (see k_gamma_hat).
void launch_gamma_hat(cudaStream_t st, bool ff, const double* gamma, int m, const int4* relk,
                      const int4* relc, const int* itrmo, int i0, int nij, double* out);
// The same operand transposed to float-float rows of length ldk (split path).
void launch_gamma_hat_t(cudaStream_t st, const double* gamma, int m, const int4* relk,
                        const int4* relc, const int* itrmo, int i0, int nij, long long ldk,
                        double* out);
// acc[i] += sum_b part[b * len + i] (FP64 or float-float partials)
void launch_partial_sum(cudaStream_t st, bool ff, const double* part, int nb, long long len,
                        double* acc);

// ---- tmoone's skeleton Fock build (rt_fock.cu) ----
struct FockRec {       // a chunk of one integral record of files 1..MFIL
    long long off, nt; // first integral in the resident arrays, count
    int it, pad;       // integral type 1..14
};
// fock[s][x][T] += terms of every integral of recs (nmat density sets of
// four arrays AAR, BAR, AAI, BAI of nsc(nsc+1)/2 elements): FOCK's terms, or
// with gaunt GAUNT's (types 2, 10, 11, 13, 14 only).  A label outside
// 1..nsc sets *bad and the integral is skipped.
void launch_fock_skeleton(cudaStream_t st, bool gaunt, const double* rint, const int* l2, const int* l1,
                          const FockRec* recs, int nrec, int nsc, int nmat, const double* dens,
                          double* fock, unsigned long long* bad);

}  // namespace rt
