// rt_kernels.cu -- device kernels of the plain transformation path:
// record scatter, FP64 GEMM, the Kramers selection / transpose between the
// two half-transformations, the symmetric expansion of the half-transformed
// integrals, and the MDCINT element selection and compaction.
#include <map>
#include <mutex>
#include <cuda_runtime.h>
#include <stdint.h>

#include "rt_ff.cuh"
#include "rt_kernels.h"

namespace rt {

// GETTW's factor for integral type it (gettw.F:33-45).
__device__ __forceinline__ double gettw_factor(int it) {
    if (it == 1) return 0.125;
    if (it == 2) return 0.5;
    if (it == 3) return 0.25;
    if (it <= 8) return 0.5;
    return 1.0;
}

// ---------------------------------------------------------------------------
// FP64 GEMM, C = A(MxK, row-major) * B(KxN, row-major), batched over
// blockIdx.z; the epilogue functor places each element.
// ---------------------------------------------------------------------------

template <class Epi>
__global__ void __launch_bounds__(256) k_gemm_f64(const double* __restrict__ A, long long lda,
                                                  long long sA, const double* __restrict__ B,
                                                  long long ldb, long long sB, int M, int N, int K,
                                                  int mx, Epi epi) {
    __shared__ double As[16][65];
    __shared__ double Bs[16][64];
    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int bz = blockIdx.z;
    const double* Ab = A + (long long)bz * sA;
    const double* Bb = B + (long long)bz * sB;
    // the larger of the two tile counts runs along grid.x (no 65535 limit)
    const int m0 = (mx ? blockIdx.x : blockIdx.y) * 64, n0 = (mx ? blockIdx.y : blockIdx.x) * 64;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    const int ar = t >> 2, ak = (t & 3) * 4;
    const int bk = t >> 4, bn = (t & 15) * 4;
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int row = m0 + ar;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int k = k0 + ak + u;
            As[ak + u][ar] = (row < M && k < K) ? Ab[(long long)row * lda + k] : 0.0;
        }
        const int kk = k0 + bk;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int col = n0 + bn + u;
            Bs[bk][bn + u] = (kk < K && col < N) ? Bb[(long long)kk * ldb + col] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[q][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[q][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int row = m0 + tx + 16 * i, col = n0 + ty + 16 * j;
            if (row < M && col < N) epi(bz, row, col, acc[i][j]);
        }
}

template <class Epi>
void gemm_f64(cudaStream_t st, const double* A, long long lda, long long sA, const double* B,
              long long ldb, long long sB, int M, int N, int K, int batch, Epi epi) {
    const unsigned tm = (M + 63) / 64, tn = (N + 63) / 64;
    const int mx = tm > tn;
    dim3 grid(mx ? tm : tn, mx ? tn : tm, batch);
    if (grid.y > 65535u || grid.z > 65535u) throw_dim("GEMM grid too large");
    k_gemm_f64<Epi><<<grid, 256, 0, st>>>(A, lda, sA, B, ldb, sB, M, N, K, mx, epi);
}

template void gemm_f64<EpiHA>(cudaStream_t, const double*, long long, long long, const double*,
                              long long, long long, int, int, int, int, EpiHA);
template void gemm_f64<EpiRowMajor>(cudaStream_t, const double*, long long, long long,
                                    const double*, long long, long long, int, int, int, int,
                                    EpiRowMajor);
template void gemm_f64<EpiRK>(cudaStream_t, const double*, long long, long long, const double*,
                              long long, long long, int, int, int, int, EpiRK);

// Element formats of the intermediate arrays: FP64 (plain path) and
// float-float (split path).  comb(a, b, sg) = a + sg*b.
// magnitude of the complex number a + ib in FP32 without underflow of the squares
__device__ __forceinline__ float mag32(float a, float b) {
    a = fabsf(a);
    b = fabsf(b);
    const float mx = fmaxf(a, b), mn = fminf(a, b);
    if (mx == 0.f) return 0.f;
    const float r = __fdividef(mn, mx);
    return mx * sqrtf(fmaf(r, r, 1.f));
}

// Threshold tests: |re + i im| compared with a threshold, in FP64 on the
// plain path, in FP32 on the leading parts on the split path (the float-float
// values carry their magnitude in .x; FP64 arithmetic runs at about 1/70 of
// the FP32 rate on GB300).
struct F64El {
    typedef double T;
    static __device__ __forceinline__ T comb(T a, T b, double sg) { return a + sg * b; }
    static __device__ __forceinline__ T neg(T a) { return -a; }
    static __device__ __forceinline__ double mag(T re, T im) { return hypot(re, im); }
    // a part of magnitude at most thr is not stored (trbout.F:61-115)
    static __device__ __forceinline__ T keep(T a, double thr) { return fabs(a) > thr ? a : 0.0; }
    static __device__ __forceinline__ double val(T a) { return a; }
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T from(double v) { return v; }
    static __device__ __forceinline__ bool nonzero(T re, T im) { return re != 0.0 || im != 0.0; }
    static __device__ __forceinline__ bool above(T re, T im, double thr) { return hypot(re, im) > thr; }
    // TROUT's screen (trout.F:30-43): kept unless VMX product or value too small
    static __device__ __forceinline__ bool screen(T re, T im, double vv, float, double thrgen) {
        return !(vv < thrgen) && !(hypot(re, im) < thrgen / vv);
    }
};
struct FFEl {
    typedef float2 T;
    static __device__ __forceinline__ T comb(T a, T b, double sg) { return ff_add(a, b, (float)sg); }
    static __device__ __forceinline__ T neg(T a) { return make_float2(-a.x, -a.y); }
    static __device__ __forceinline__ double mag(T re, T im) { return (double)mag32(re.x, im.x); }
    static __device__ __forceinline__ T keep(T a, double thr) {
        return fabsf(a.x) > (float)thr ? a : make_float2(0.f, 0.f);
    }
    static __device__ __forceinline__ double val(T a) { return ff_to_double(a); }
    static __device__ __forceinline__ T zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ bool nonzero(T re, T im) { return re.x != 0.f || im.x != 0.f; }
    static __device__ __forceinline__ bool above(T re, T im, double thr) {
        return mag32(re.x, im.x) > (float)thr;
    }
    static __device__ __forceinline__ bool screen(T re, T im, double, float thr, double) {
        return !(mag32(re.x, im.x) < thr);
    }
    static __device__ __forceinline__ T from(double v) {
        const float h = __double2float_rn(v);
        return make_float2(h, __double2float_rn(v - (double)h));
    }
};

// ---------------------------------------------------------------------------
// K2: Kramers-unique selection + time-reversal completion + transpose
// (MTIMHER + TROUT + SR2FLSH + GETHTI + UNIQUE: mtimher.F:3-26,
// trout.F:1-63, unique.F:1-50).  With the full symmetric G_pq the
// half-transformed integral of the pair (I, J) is
//   (pq| I J) = RI(I,J) + s_IJ RI(Jbar, Ibar),   s_IJ = sign(ITRMO(I) ITRMO(J)),
// RI = QA^H G_pq QA.  The screening test of TROUT (trout.F:30-43) is
// applied to these values.
// ---------------------------------------------------------------------------
// pair_thr: THRGEN / VMX(p) VMX(q) per pair (+inf where the product is below
// THRGEN), the threshold of the split path's FP32 test.
template <class E>
__global__ void k_tr_select(const typename E::T* __restrict__ ri, int m, int npc, int pq0, int P,
                            const int4* __restrict__ items, const float* __restrict__ item_sign,
                            int it0, int nitems, const double* __restrict__ pair_vmx,
                            const float* __restrict__ pair_thr, double thrgen,
                            typename E::T* __restrict__ hp, unsigned long long* __restrict__ kept) {
    typedef typename E::T T;
    const int it = it0 + blockIdx.y;
    const int pql = blockIdx.x * blockDim.x + threadIdx.x;
    int keep = 0;
    if (pql < npc && it < nitems) {
        const int4 w = items[it];  // I, J, Ibar, Jbar (0-based spinors)
        const double s = item_sign[it];
        const long long plane = (long long)m * m * npc;
        const long long a = ((long long)w.x * m + w.y) * npc + pql;
        const long long b = ((long long)w.w * m + w.z) * npc + pql;
        T re = E::comb(ri[a], ri[b], s);
        T im = E::comb(ri[plane + a], ri[plane + b], s);
        const int pq = pq0 + pql;
        const bool pass = E::screen(re, im, pair_vmx[pq], pair_thr ? pair_thr[pq] : 0.f, thrgen);
        if (!pass) { re = E::zero(); im = E::zero(); }
        keep = pass && E::nonzero(re, im);
        const long long o = (long long)it * P + pq;
        hp[o] = re;
        hp[(long long)nitems * P + o] = im;
    }
    keep = __syncthreads_count(keep);
    if (threadIdx.x == 0 && keep) atomicAdd(kept, (unsigned long long)keep);
}

// ---------------------------------------------------------------------------
// Gaunt (Breit) selection: the three half-transformed streams TRBOUT stores
// for the Kramers-unique pair (I', J') that UNIQUE (with the Breit sign,
// unique.F:34) gives for TRANS2's item (I, J), transformed as TRANS2 does
// (conjugate and swap the QB streams, negate: trans2.F:129-155):
//   A = HA(J',I'),  B = HB(J',I'),  C = conj(HB(I',J')),
//   HA(x,y) = RIA(x,y) + s RIA(ybar,xbar)   (MTIMHER with ISG = -1)
//   HB(x,y) = RI2(x,y) + s RI2(ybar,xbar)   (MTIMHR2), s = -sign(ITRMO(x) ITRMO(y)),
// RIA = QA^H G QA over the whole pair block, RI2 = QB^H G QA over its
// small-component rows.  TRBOUT's fixed screen: nothing is kept when
// |A| + |B| + |HB(I',J')| < 1e-16, and parts of magnitude at most 1e-16 are
// zero (trbout.F:35-115).  Output: three streams [stream][plane][item][pair].
// ---------------------------------------------------------------------------
template <class E>
__global__ void k_trb_select(const typename E::T* __restrict__ ria, const typename E::T* __restrict__ ri2,
                             int m, int npc, int pq0, int P, const BreitItem* __restrict__ items, int it0,
                             int nitems, typename E::T* __restrict__ hp, unsigned long long* __restrict__ kept) {
    typedef typename E::T T;
    const int it = it0 + blockIdx.y;
    const int pql = blockIdx.x * blockDim.x + threadIdx.x;
    int keep = 0;
    if (pql < npc && it < nitems) {
        const BreitItem w = items[it];
        const double s = w.s;
        const long long plane = (long long)m * m * npc;
        auto at = [&](int a, int b) { return ((long long)a * m + b) * npc + pql; };
        const long long xy = at(w.x, w.y), yx = at(w.y, w.x), ybxb = at(w.yb, w.xb), xbyb = at(w.xb, w.yb);
        T ar = E::comb(ria[xy], ria[ybxb], s), ai = E::comb(ria[plane + xy], ria[plane + ybxb], s);
        T br = E::comb(ri2[xy], ri2[ybxb], s), bi = E::comb(ri2[plane + xy], ri2[plane + ybxb], s);
        T cr = E::comb(ri2[yx], ri2[xbyb], s), ci = E::comb(ri2[plane + yx], ri2[plane + xbyb], s);
        const double TB = 1.0e-16;
        if (E::mag(ar, ai) + E::mag(br, bi) + E::mag(cr, ci) < TB) {
            ar = ai = br = bi = cr = ci = E::zero();
        } else {
            keep = 1;
            ar = E::keep(ar, TB); ai = E::keep(ai, TB);
            br = E::keep(br, TB); bi = E::keep(bi, TB);
            cr = E::keep(cr, TB); ci = E::neg(E::keep(ci, TB));  // C = conj(HB(I',J'))
        }
        if (w.conj) {  // conjugate all three, swap B and C
            T tr = cr, ti = ci;
            ai = E::neg(ai);
            cr = br; ci = E::neg(bi);
            br = tr; bi = E::neg(ti);
        }
        if (w.neg) {
            ar = E::neg(ar); ai = E::neg(ai);
            br = E::neg(br); bi = E::neg(bi);
            cr = E::neg(cr); ci = E::neg(ci);
        }
        const long long o = (long long)it * P + pq0 + pql, st = 2LL * nitems * P, pl = (long long)nitems * P;
        hp[o] = ar; hp[pl + o] = ai;
        hp[st + o] = br; hp[st + pl + o] = bi;
        hp[2 * st + o] = cr; hp[2 * st + pl + o] = ci;
    }
    keep = __syncthreads_count(keep);
    if (threadIdx.x == 0 && keep) atomicAdd(kept, (unsigned long long)keep);
}

// ---------------------------------------------------------------------------
// Symmetric expansion of the half-transformed integrals of one component
// block (the role of MATMUL3's two updates, matmul3.F:25-32):
//   M3[p][ij][plane][q] = Hp[plane][ij][pair(p,q)]
// ---------------------------------------------------------------------------
// The row blocks of one item are adjacent in launch order (blockIdx.x), so
// the item's half-transformed row stays in L2 while they gather from it.
// Rows p of one component against columns q of the same component
// (Coulomb) or of the other one (Gaunt: M(p,q) = M(q,p) = H(pq), p and q in
// different components); `two` doubles the values (MATMUL7's factor 2,
// matmul7.F:3-35; exact, also on float-float pairs).
template <bool FF>
__global__ void k_expand(const double* __restrict__ hp, int P, int nitems, int it0, int nij,
                         const int* __restrict__ pidx, int nrow, int ncol, bool two, bool diag2,
                         double* __restrict__ m3) {
    const int ijl = blockIdx.y;
    const int it = it0 + ijl;
    const double* hr = hp + (long long)it * P;
    const double* hi = hp + (long long)nitems * P + (long long)it * P;
    for (int p = blockIdx.x; p < nrow; p += gridDim.x) {
        double* row = m3 + ((long long)p * nij + ijl) * (2LL * ncol);
        for (int q = threadIdx.x; q < ncol; q += blockDim.x) {
            int pq = pidx[p * ncol + q];
            double re = 0.0, im = 0.0;
            if (pq >= 0) { re = hr[pq]; im = hi[pq]; }
            // x2 (MATMUL7) and x2 on the diagonal of rotran's half buckets
            // (MATMUL3's two updates of p = q): exact, also on FF halves
            const int e = (two ? 1 : 0) + (diag2 && p == q ? 1 : 0);
            if (e) {
                if (FF) {
                    const float f = e == 2 ? 4.f : 2.f;
                    float2 a = *reinterpret_cast<float2*>(&re), b = *reinterpret_cast<float2*>(&im);
                    a.x *= f; a.y *= f; b.x *= f; b.y *= f;
                    re = *reinterpret_cast<double*>(&a);
                    im = *reinterpret_cast<double*>(&b);
                } else {
                    const double f = e == 2 ? 4.0 : 2.0;
                    re *= f;
                    im *= f;
                }
            }
            row[q] = re;
            row[ncol + q] = im;
        }
    }
}

// ---------------------------------------------------------------------------
// MDCINT element selection (MSUMTIM + OUTPP1/OUTPP2 + PPSYM:
// msumtim.F:3-21, outpp1.F:1-74, outpp2.F:1-139, ppsym.F:67-91).
// One block per record; positions (KKR, LKR) in the order PPSYM writes them;
// an element is written when it belongs to the record's canonical set and
// |value| > THROUT.  The value is the complete integral
//   RL(K,L) = RLR(K,L) + s_KL RLR(Lbar,Kbar).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool in_set(int cls, int x, int y, int i, int j) {
    // x, y, i, j 1-based Kramers indices; cls 0..3 = MDCINT classes 1..4
    if (cls == 3) return true;
    if (cls == 0) {
        if (i == j) return y <= x && x <= i;
        int a = x > y ? x : y, b = x > y ? y : x;
        return a < i || (a == i && b <= j);
    }
    return y <= x && (x < i || (x == i && y <= j));
}

// mode 0 counts the elements of each record, mode 1 writes them at the
// offsets produced by k_scan_records; both evaluate the same expressions.
template <class E>
__global__ void __launch_bounds__(256) k_emit(const typename E::T* __restrict__ rlr, int m, int nij,
                                              int K, const EmitRec* __restrict__ rec,
                                              const int* __restrict__ kra,
                                              const int* __restrict__ krb,
                                              const int* __restrict__ itrmo, double throut,
                                              int mode, OutStreams os) {
    __shared__ int wsum[8];
    __shared__ int base;
    const EmitRec R = rec[blockIdx.x];
    const int ijl = R.ijl, cls = R.cls, i = R.ikr, j = R.jkr;
    const int ks = (cls == 2 || cls == 3) ? 1 : -1;   // class signs (rotran.F:306-328)
    const int ls = (cls == 1 || cls == 3) ? 1 : -1;
    const long long plane = (long long)m * nij * m;
    long long dst = 0;
    if (mode == 1) dst = os.off[cls][R.rank];
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int KK = K * K;
    for (int t0 = 0; t0 < KK; t0 += blockDim.x) {
        const int pos = t0 + threadIdx.x;
        bool emit = false;
        double re = 0.0, im = 0.0;
        int x = 0, y = 0;
        if (pos < KK) {
            x = pos / K + 1;
            y = pos - (x - 1) * K + 1;
            typename E::T vr = E::zero(), vi = E::zero();
            if (in_set(cls, x, y, i, j)) {
                const int Ks = (ks < 0 ? krb[x - 1] : kra[x - 1]) - 1;
                const int Ls = (ls < 0 ? krb[y - 1] : kra[y - 1]) - 1;
                const int Kb = abs(itrmo[Ks]) - 1, Lb = abs(itrmo[Ls]) - 1;
                const double sg = ((itrmo[Ks] > 0) == (itrmo[Ls] > 0)) ? 1.0 : -1.0;
                const long long a = ((long long)Ks * nij + ijl) * m + Ls;
                const long long b = ((long long)Lb * nij + ijl) * m + Kb;
                vr = E::comb(rlr[a], rlr[b], sg);
                vi = E::comb(rlr[plane + a], rlr[plane + b], sg);
            }
            emit = E::above(vr, vi, throut);
            if (emit && mode == 1) {  // FP64 values only for the elements written
                re = E::val(vr);
                im = E::val(vi);
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, emit);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        int off = base, tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            if (w < warp) off += wsum[w];
            tot += wsum[w];
        }
        off += __popc(bal & ((1u << lane) - 1u));
        if (emit && mode == 1) {
            const long long o = dst + off;
            os.idx[cls][2 * o] = x * ks;
            os.idx[cls][2 * o + 1] = y * ls;
            os.val[cls][2 * o] = re;
            os.val[cls][2 * o + 1] = im;
        }
        __syncthreads();
        if (threadIdx.x == 0) base += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && mode == 0) os.cnt[cls][R.rank] = base;
}

// ---------------------------------------------------------------------------
// Records from rotran's two halves.  rotran's TRANS1 buckets each integral
// under its LABEL1 pair only (sort1.F:78-142), so the value RL_IJ(K,L) that
// TRANS2 forms for item (I, J) is half of an integral; PPSYM adds the other
// half, pushed by OUTPP2 from the item whose Kramers indices are the
// element's (ppsym.F:67-91, outpp2.F:1-139).  For the Gaunt integrals
// (MSUMTIM with ISG = -1 plus the two MATMUL7 streams, trans2.F:129-177) the
// two halves are not related by a symmetry of the item's own result, so all
// items' RL are kept (rl_all) and each element is assembled as PPSYM does:
//   OUTPP1's part of the record's item (outpp1.F:1-74: loop 1 at (x, y),
//   loop 2 at the transposed position for classes 1 and 4), plus
//   OUTPP2's loop-1 part of item (x, y) when the record lies in that item's
//   range, plus its loop-2 part (conjugated, classes 1 and 4) of item (y, x);
// each part is kept only above THROUT, as OUTPP1/OUTPP2 test it (outpp1.F:34,
// outpp2.F:40), and the sum is tested again as PPSYM does.  Classes 3 and 4
// push CJVEC / CJNVEC images of RL (trans2.F:284-303).  The Coulomb
// transform takes this path on request (rotran's exact intermediate).
// ---------------------------------------------------------------------------
template <class E>
__global__ void k_rl_store(const typename E::T* __restrict__ rlr, const typename E::T* __restrict__ rlr_b,
                           const typename E::T* __restrict__ rlr_c, int m, int nij, int it0,
                           const int* __restrict__ itrmo, double isg, double2* __restrict__ rl_all) {
    const int ijl = blockIdx.y;
    const long long plane = (long long)m * nij * m;
    for (int kl = blockIdx.x * blockDim.x + threadIdx.x; kl < m * m; kl += gridDim.x * blockDim.x) {
        const int k = kl / m, l = kl - k * m;
        const int kb = abs(itrmo[k]) - 1, lb = abs(itrmo[l]) - 1;
        const double sg = ((itrmo[k] > 0) == (itrmo[l] > 0)) ? isg : -isg;
        const long long a = ((long long)k * nij + ijl) * m + l;
        const long long b = ((long long)lb * nij + ijl) * m + kb;
        typename E::T vr = E::comb(rlr[a], rlr[b], sg), vi = E::comb(rlr[plane + a], rlr[plane + b], sg);
        if (rlr_b) {
            vr = E::comb(E::comb(vr, rlr_b[a], 1.0), rlr_c[a], 1.0);
            vi = E::comb(E::comb(vi, rlr_b[plane + a], 1.0), rlr_c[plane + a], 1.0);
        }
        rl_all[((long long)(it0 + ijl) * m + k) * m + l] = make_double2(E::val(vr), E::val(vi));
    }
}

// one half of an element, kept when above THROUT
__device__ __forceinline__ void add_half(double& re, double& im, double2 v, double throut) {
    if (hypot(v.x, v.y) > throut) { re += v.x; im += v.y; }
}

__global__ void __launch_bounds__(256) k_emit_halves(const double2* __restrict__ rl_all, int m, int K, int it0,
                                                    const EmitRec* __restrict__ rec,
                                                    const int* __restrict__ item_of,
                                                    const int* __restrict__ kra, const int* __restrict__ krb,
                                                    double throut, int mode, OutStreams os) {
    __shared__ int wsum[8];
    __shared__ int base;
    const EmitRec R = rec[blockIdx.x];
    const int c = R.cls + 1, a = R.ikr, b = R.jkr;  // class 1..4, record (a, b), 1-based
    const double2* own = rl_all + (long long)(it0 + R.ijl) * m * m;
    // spinor tables of OUTPP1 (krk1, krl1) and OUTPP2 (krk2, krl2) per class
    const int* krk1 = (c == 3 || c == 4) ? kra : krb;
    const int* krl1 = (c == 2 || c == 4) ? kra : krb;
    const int* krk2 = (c == 3 || c == 4) ? kra : krb;
    const int* krl2 = c == 2 ? kra : krb;
    const int* pitem = item_of + ((c == 1 || c == 4) ? 1 : 0) * K * K;  // pushing items: J barred for 1, 4
    const int ks = (c == 3 || c == 4) ? 1 : -1;                            // element label signs
    const int ls = (c == 2 || c == 4) ? 1 : -1;                            // (rotran.F:306-328)
    long long dst = 0;
    if (mode == 1) dst = os.off[R.cls][R.rank];
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int KK = K * K;
    // the pushed image of an item's RL: RL, conj (CJVEC), -conj (CJNVEC)
    auto pushed = [&](double2 v) {
        if (c == 3) return make_double2(v.x, -v.y);
        if (c == 4) return make_double2(-v.x, v.y);
        return v;
    };
    for (int t0 = 0; t0 < KK; t0 += blockDim.x) {
        const int pos = t0 + threadIdx.x;
        bool emit = false;
        double re = 0.0, im = 0.0;
        int x = 0, y = 0;
        if (pos < KK) {
            x = pos / K + 1;
            y = pos - (x - 1) * K + 1;
            const int xmax = c == 4 ? K : a;
            // OUTPP1 loop 1 at (x, y)
            if (x <= xmax && y <= ((c <= 3 && x == a) ? b : x))
                add_half(re, im, own[(long long)(krk1[x - 1] - 1) * m + krl1[y - 1] - 1], throut);
            // OUTPP1 loop 2: position (y', x') = (x, y)
            if ((c == 1 && a != b) || c == 4) {
                const int xp = y, yp = x;
                if (xp <= xmax) {
                    int ym = (c <= 3 && xp == a) ? b : xp;
                    if (ym == xp) --ym;
                    if (yp <= ym)
                        add_half(re, im, own[(long long)(krl1[yp - 1] - 1) * m + krk1[xp - 1] - 1], throut);
                }
            }
            // OUTPP2 loop 1 of item (x, y)
            if (y <= x) {
                const int kmin = c == 4 ? 1 : x, lmin = (c <= 3 && a == x) ? y : 1;
                const int t = pitem[(x - 1) * K + (y - 1)];
                if (t >= 0 && a >= kmin && b >= lmin && b <= a)
                    add_half(re, im, pushed(rl_all[((long long)t * m + krk2[a - 1] - 1) * m + krl2[b - 1] - 1]),
                             throut);
            }
            // OUTPP2 loop 2 of item (y, x), conjugated, at position (x, y)
            if (x < y && (c == 1 || c == 4)) {
                const int i = y, j = x;
                const int kmin = c == 4 ? 1 : i, lmin = (c <= 3 && a == i) ? j : 1;
                const int t = pitem[(i - 1) * K + (j - 1)];
                if (t >= 0 && a >= kmin && b >= lmin && b <= a - 1) {
                    const double2 v =
                        pushed(rl_all[((long long)t * m + krl2[b - 1] - 1) * m + krk2[a - 1] - 1]);
                    add_half(re, im, make_double2(v.x, -v.y), throut);
                }
            }
            // the positions OUTPP1/OUTPP2 reach are the canonical set, which
            // also bounds the record's output (all K*K with THROUT < 0)
            emit = (throut < 0.0 || in_set(R.cls, x, y, a, b)) && hypot(re, im) > throut;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, emit);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        int off = base, tot = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            if (w < warp) off += wsum[w];
            tot += wsum[w];
        }
        off += __popc(bal & ((1u << lane) - 1u));
        if (emit && mode == 1) {
            const long long o = dst + off;
            os.idx[R.cls][2 * o] = x * ks;
            os.idx[R.cls][2 * o + 1] = y * ls;
            os.val[R.cls][2 * o] = re;
            os.val[R.cls][2 * o + 1] = im;
        }
        __syncthreads();
        if (threadIdx.x == 0) base += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0 && mode == 0) os.cnt[R.cls][R.rank] = base;
}

// Exclusive scan of the element counts of one chunk's records, per class,
// continuing from the running class totals in os.total (single block).
__global__ void __launch_bounds__(1024) k_scan_records(const EmitRec* __restrict__ rec, int nrec,
                                                       OutStreams os) {
    __shared__ long long part[1024][4];
    const int t = threadIdx.x, nt = blockDim.x;
    const int per = (nrec + nt - 1) / nt;
    const int r0 = t * per, r1 = min(nrec, r0 + per);
    long long s[4] = {0, 0, 0, 0};
    for (int r = r0; r < r1; ++r) s[rec[r].cls] += os.cnt[rec[r].cls][rec[r].rank];
    for (int c = 0; c < 4; ++c) part[t][c] = s[c];
    __syncthreads();
    if (t < 4) {  // serial scan over the 1024 partial sums of class t
        long long run = os.total[t];
        for (int q = 0; q < nt; ++q) {
            long long v = part[q][t];
            part[q][t] = run;
            run += v;
        }
        os.total[t] = run;
    }
    __syncthreads();
    long long o[4] = {part[t][0], part[t][1], part[t][2], part[t][3]};
    for (int r = r0; r < r1; ++r) {
        const int c = rec[r].cls;
        os.off[c][rec[r].rank] = o[c];
        o[c] += os.cnt[c][rec[r].rank];
    }
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------
void launch_tr_select(cudaStream_t st, bool ff, const double* ri, int m, int npc, int pq0, int P,
                      const int4* items, const float* item_sign, int nitems,
                      const double* pair_vmx, const float* pair_thr, double thrgen, double* hp,
                      unsigned long long* kept) {
    for (int y0 = 0; y0 < nitems; y0 += 65535) {
        int ny = nitems - y0 < 65535 ? nitems - y0 : 65535;
        dim3 grid((npc + 255) / 256, ny);
        if (ff)
            k_tr_select<FFEl><<<grid, 256, 0, st>>>((const float2*)ri, m, npc, pq0, P, items,
                                                   item_sign, y0, nitems, pair_vmx, pair_thr,
                                                   thrgen, (float2*)hp, kept);
        else
            k_tr_select<F64El><<<grid, 256, 0, st>>>(ri, m, npc, pq0, P, items, item_sign, y0,
                                                    nitems, pair_vmx, nullptr, thrgen, hp, kept);
    }
}

void launch_expand(cudaStream_t st, const double* hp, int P, int nitems, int it0, int nij,
                   const int* pidx, int nrow, int ncol, double* m3, bool two, bool ff, bool diag2) {
    if (nij > 65535) throw_dim("expansion: more than 65535 items per chunk");
    if (nrow <= 0 || ncol <= 0) return;
    dim3 grid(nrow < 64 ? nrow : 64, nij);
    if (ff) k_expand<true><<<grid, 128, 0, st>>>(hp, P, nitems, it0, nij, pidx, nrow, ncol, two, diag2, m3);
    else k_expand<false><<<grid, 128, 0, st>>>(hp, P, nitems, it0, nij, pidx, nrow, ncol, two, diag2, m3);
}

void launch_trb_select(cudaStream_t st, bool ff, const double* ria, const double* ri2, int m, int npc,
                       int pq0, int P, const BreitItem* items, int nitems, double* hp,
                       unsigned long long* kept) {
    for (int y0 = 0; y0 < nitems; y0 += 65535) {
        int ny = nitems - y0 < 65535 ? nitems - y0 : 65535;
        dim3 grid((npc + 255) / 256, ny);
        if (ff)
            k_trb_select<FFEl><<<grid, 256, 0, st>>>((const float2*)ria, (const float2*)ri2, m, npc, pq0, P,
                                                    items, y0, nitems, (float2*)hp, kept);
        else
            k_trb_select<F64El><<<grid, 256, 0, st>>>(ria, ri2, m, npc, pq0, P, items, y0, nitems, hp, kept);
    }
}

void launch_emit(cudaStream_t st, bool ff, const double* rlr, int m, int nij, int K,
                 const EmitRec* rec, int nrec, const int* kra, const int* krb, const int* itrmo,
                 double throut, const OutStreams& os) {
    if (nrec <= 0) return;
    for (int mode = 0; mode < 2; ++mode) {
        if (mode == 1) k_scan_records<<<1, 1024, 0, st>>>(rec, nrec, os);
        if (ff)
            k_emit<FFEl><<<nrec, 256, 0, st>>>((const float2*)rlr, m, nij, K, rec, kra, krb, itrmo,
                                              throut, mode, os);
        else
            k_emit<F64El><<<nrec, 256, 0, st>>>(rlr, m, nij, K, rec, kra, krb, itrmo, throut, mode, os);
    }
}

void launch_rl_store(cudaStream_t st, bool ff, const double* rlr, const double* rlr_b, const double* rlr_c,
                     int m, int nij, int it0, const int* itrmo, double isg, double* rl_all) {
    if (nij <= 0) return;
    if (nij > 65535) throw_dim("item chunk too large for the RL store grid");
    dim3 grid((m * m + 255) / 256, nij);
    if (ff)
        k_rl_store<FFEl><<<grid, 256, 0, st>>>((const float2*)rlr, (const float2*)rlr_b, (const float2*)rlr_c, m,
                                                nij, it0, itrmo, isg, (double2*)rl_all);
    else
        k_rl_store<F64El><<<grid, 256, 0, st>>>(rlr, rlr_b, rlr_c, m, nij, it0, itrmo, isg, (double2*)rl_all);
}

void launch_emit_halves(cudaStream_t st, const double* rl_all, int m, int K, int it0, const EmitRec* rec,
                        int nrec, const int* item_of, const int* kra, const int* krb, double throut,
                        const OutStreams& os) {
    if (nrec <= 0) return;
    for (int mode = 0; mode < 2; ++mode) {
        if (mode == 1) k_scan_records<<<1, 1024, 0, st>>>(rec, nrec, os);
        k_emit_halves<<<nrec, 256, 0, st>>>((const double2*)rl_all, m, K, it0, rec, item_of, kra, krb, throut,
                                            mode, os);
    }
}

}  // namespace rt

// ===========================================================================
// pq buckets of the integral records (the role of SORT1 + INTSRT + GETSTI:
// sort1.F:70-163, getsti.F:1-49) and their expansion into the GEMM1
// operand, one pair chunk at a time
// ===========================================================================
namespace rt {

// rank of this lane among the active lanes with the same key, after one
// atomic per distinct key and warp
__device__ __forceinline__ long long warp_agg_add(int* counter, int key, bool active) {
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (mask == 0u) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    const int lkey = __shfl_sync(0xffffffffu, key, leader);
    // common case of integrals sharing their first pair: one atomic per warp
    if (__all_sync(0xffffffffu, !active || key == lkey)) {
        int base = 0;
        if (lane == leader) base = atomicAdd(&counter[key], __popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        return active ? (long long)base + __popc(mask & ((1u << lane) - 1u)) : -1;
    }
    return active ? (long long)atomicAdd(&counter[key], 1) : -1;
}

// Decode integral x; returns the number of pq bucket entries (0..2) with
// their pq buckets and packed (r, s) labels and the value.
// record holding integral x (binary search over the record offsets)
__device__ __forceinline__ int find_record(long long x, const long long* __restrict__ rec_off,
                                           int nrec) {
    int lo = 0, hi = nrec - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (rec_off[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// warp strips of 32 integrals each thread of the record scans takes at once
constexpr int SCAN_U = 2;

// Record of integral x for a warp handling 32 consecutive integrals: one
// search by the first lane, shared when the whole warp lies in that record.
__device__ __forceinline__ int warp_record(long long x, long long x0, long long nint,
                                           const long long* __restrict__ rec_off, int nrec) {
    int r0 = 0;
    if ((threadIdx.x & 31) == 0) r0 = find_record(x0, rec_off, nrec);
    r0 = __shfl_sync(0xffffffffu, r0, 0);
    const long long end = r0 + 1 < nrec ? rec_off[r0 + 1] : nint;
    if (__all_sync(0xffffffffu, x >= nint || x < end)) return r0;
    return x < nint ? find_record(x, rec_off, nrec) : r0;
}

// The record words of one integral, loaded ahead of its decoding.
struct RecWords {
    double v;
    int L2, L1;
};

__device__ __forceinline__ RecWords load_words(long long x, long long nint, const double* __restrict__ rint,
                                               const int* __restrict__ l2, const int* __restrict__ l1) {
    RecWords w{0.0, 0, 0};
    if (x < nint) {
        w.v = rint[x];
        w.L2 = l2[x];
        w.L1 = l1[x];
    }
    return w;
}

__device__ __forceinline__ int decode_integral(const RecWords& w, int rec, const int2* __restrict__ rec_meta,
                                               const ScatterTabs& tb, unsigned int* status,
                                               int* pqs, int* rss, double& v) {
    const int2 meta = rec_meta[rec];
    // SORT1 reads files 1..MFIL, or file 4 alone for the Gaunt integrals (sort1.F:55-57)
    if (tb.breit ? meta.x != 4 : (meta.x < 1 || meta.x > tb.mfil)) return 0;
    const int L2 = w.L2, L1 = w.L1;
    int a = (L2 >> 16) & 0xFFFF, b = L2 & 0xFFFF;
    int c = (L1 >> 16) & 0xFFFF, d = L1 & 0xFFFF;
    if (a < 1 || b < 1 || c < 1 || d < 1 || a > tb.n || b > tb.n || c > tb.n || d > tb.n || d > c) {
        atomicOr(status, ST_BAD_LABEL);
        return 0;
    }
    --a; --b; --c; --d;
    const int pa = a > b ? a : b, pb = a > b ? b : a;
    const int cdo = c * (c + 1) / 2 + d;
    if (!tb.pq_read[cdo]) return 0;  // INDPQ(pq) == 0: never transformed
    const int coinc = (pa == pb) + (c == d) + (pa == c && pb == d);
    // Complete sums: the unique integral under both pairs (its full symmetric
    // form).  Half buckets: rotran's entry, under LABEL1's pair only with
    // GETTW's factor as it is; r = s counts twice, as MTIMHER's transposed
    // orientation counts it (mtimher.F:3-26), which the symmetric storage of
    // G_pq holds once (p = q is doubled after TROUT's screen, in k_expand,
    // as MATMUL3's second update does).  The records add the
    // pair-interchanged half (k_emit_halves).  GETTW turns the sign of the
    // Gaunt file (gettw.F:51-55).
    v = w.v * gettw_factor(meta.y) * (tb.half ? (pa == pb ? 2.0 : 1.0) : (double)(1 << coinc));
    if (tb.breit) v = -v;
    const int abo = pa * (pa + 1) / 2 + pb;
    int ne = 0;
    for (int dir = 0; dir < 2; ++dir) {
        if (dir == 1 && (abo == cdo || tb.half)) break;
        const int pq = tb.pair_of_orig[dir == 0 ? cdo : abo];
        const int r = dir == 0 ? pa : c, s = dir == 0 ? pb : d;
        if (pq < 0) { atomicOr(status, ST_BAD_BLOCK); return 0; }
        const int pg = tb.pair_group[pq];
        const int g = tb.g1_of[pg * tb.nblk + tb.ao_block[r]];
        if (g < 0 || tb.g1_kblk[g] != tb.ao_block[s]) { atomicOr(status, ST_BAD_BLOCK); return 0; }
        if (tb.jb_base[pg * tb.nblk + tb.ao_block[s]] < 0) { atomicOr(status, ST_BAD_BLOCK); return 0; }
        pqs[ne] = pq;
        // (block, position) of r and s, and whether r == s
        rss[ne] = (int)(((unsigned)tb.ao_block[r] << 29) | ((unsigned)tb.ao_pos[r] << 17) |
                        ((unsigned)tb.ao_block[s] << 14) | ((unsigned)tb.ao_pos[s] << 2) |
                        (r == s ? 1u : 0u));
        ++ne;
    }
    return ne;
}

__global__ void __launch_bounds__(256) k_bucket_count(const double* __restrict__ rint, const int* __restrict__ l2,
                                                      const int* __restrict__ l1, long long nint,
                                                      const long long* __restrict__ rec_off,
                                                      const int2* __restrict__ rec_meta, int nrec,
                                                      ScatterTabs tb, int* __restrict__ count,
                                                      unsigned int* __restrict__ status) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long base0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
    // SCAN_U warp strips per iteration, their record words loaded together
    for (long long xb = base0; xb < nint; xb += SCAN_U * stride) {
        RecWords w[SCAN_U];
#pragma unroll
        for (int u = 0; u < SCAN_U; ++u) w[u] = load_words(xb + u * stride + (threadIdx.x & 31), nint, rint, l2, l1);
#pragma unroll
        for (int u = 0; u < SCAN_U; ++u) {
            const long long xs = xb + u * stride;  // the same for the whole warp
            if (xs >= nint) break;
            const long long x = xs + (threadIdx.x & 31);
            int pqs[2], rss[2], ne = 0;
            double v;
            const int rec = warp_record(x, xs, nint, rec_off, nrec);
            if (x < nint) ne = decode_integral(w[u], rec, rec_meta, tb, status, pqs, rss, v);
            warp_agg_add(count, ne > 0 ? pqs[0] : 0, ne > 0);
            warp_agg_add(count, ne > 1 ? pqs[1] : 0, ne > 1);
        }
    }
}

__global__ void __launch_bounds__(256) k_bucket_place(const double* __restrict__ rint, const int* __restrict__ l2,
                                                      const int* __restrict__ l1, long long nint,
                                                      const long long* __restrict__ rec_off,
                                                      const int2* __restrict__ rec_meta, int nrec,
                                                      ScatterTabs tb, const long long* __restrict__ off,
                                                      int* __restrict__ fill, double* __restrict__ bval,
                                                      int* __restrict__ brs, unsigned int* __restrict__ status) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long base0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
    for (long long xb = base0; xb < nint; xb += SCAN_U * stride) {
        RecWords w[SCAN_U];
#pragma unroll
        for (int u = 0; u < SCAN_U; ++u) w[u] = load_words(xb + u * stride + (threadIdx.x & 31), nint, rint, l2, l1);
#pragma unroll
        for (int u = 0; u < SCAN_U; ++u) {
            const long long xs = xb + u * stride;  // the same for the whole warp
            if (xs >= nint) break;
            const long long x = xs + (threadIdx.x & 31);
            int pqs[2], rss[2], ne = 0;
            double v = 0.0;
            const int rec = warp_record(x, xs, nint, rec_off, nrec);
            if (x < nint) ne = decode_integral(w[u], rec, rec_meta, tb, status, pqs, rss, v);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const long long p = warp_agg_add(fill, ne > e ? pqs[e] : 0, ne > e);
                if (ne > e) {
                    const long long o = off[pqs[e]] + p;
                    bval[o] = v;
                    brs[o] = rss[e];
                }
            }
        }
    }
}

// exclusive scan of n ints into long long offsets (single block)
__global__ void __launch_bounds__(1024) k_scan_counts(const int* __restrict__ cnt, long long n,
                                                      long long* __restrict__ off) {
    __shared__ long long part[1024];
    const int t = threadIdx.x;
    const long long per = (n + 1023) / 1024;
    const long long a = t * per, b = min(n, a + per);
    long long s = 0;
    for (long long i = a; i < b; ++i) s += cnt[i];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        long long run = 0;
        for (int q = 0; q < 1024; ++q) { long long v = part[q]; part[q] = run; run += v; }
    }
    __syncthreads();
    long long o = part[t];
    for (long long i = a; i < b; ++i) { off[i] = o; o += cnt[i]; }
    if (t == 1023) off[n] = o;
}

// Second level: one CTA per pq splits its bucket into the buckets of its
// expansion jobs, writing each element G_pq(r,s) under the job owning row r
// and, off the diagonal, G_pq(s,r) under the job owning row s, as
// (row position << 16 | column position).  The output of pq occupies
// [2 off[pq], 2 off[pq+1]); start and count of every (pq, job) bucket go to
// jstart / jcount at pg_bbase[pg] + (pq - pg start) * njobs + job.
constexpr int MAX_JOBS = 1024;
// entries each thread loads ahead in the bucket loops (memory-level parallelism)
constexpr int SPLIT_U = 4, EXPAND_U = 8;

// expansion job of a row (block, position); -1 outside the pair group's jobs
__device__ __forceinline__ int job_of(const int* jbb, const int* jbd, int nblk, int nj, int blk,
                                      int pos) {
    if (blk >= nblk || jbb[blk] < 0) return -1;
    const int j = jbb[blk] + pos / jbd[blk];
    return j < nj ? j : -1;
}

__device__ __forceinline__ int smem_agg_add(int* ctr, int key, bool active) {
    const unsigned mask = __ballot_sync(0xffffffffu, active);
    if (!active) return -1;
    const unsigned peers = __match_any_sync(mask, key);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&ctr[key], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void __launch_bounds__(256) k_bucket_split(const long long* __restrict__ off,
                                                      const double* __restrict__ bval,
                                                      const int* __restrict__ brs, ScatterTabs tb,
                                                      long long* __restrict__ jstart,
                                                      int* __restrict__ jcount,
                                                      double* __restrict__ oval,
                                                      int* __restrict__ ors) {
    __shared__ int cnt[MAX_JOBS], cur[MAX_JOBS];
    __shared__ int jbb[8], jbd[8];
    const int pq = blockIdx.x;
    const int pg = tb.pair_group[pq];
    const int nj = tb.pg_njobs[pg];
    const long long bb = tb.pg_bbase[pg] + (long long)(pq - tb.pg_start[pg]) * nj;
    for (int j = threadIdx.x; j < nj; j += blockDim.x) cnt[j] = 0;
    if (threadIdx.x < tb.nblk) {
        jbb[threadIdx.x] = tb.jb_base[pg * tb.nblk + threadIdx.x];
        jbd[threadIdx.x] = tb.jb_band[pg * tb.nblk + threadIdx.x];
    }
    __syncthreads();
    const long long e0 = off[pq], e1 = off[pq + 1];
    // the loops run in whole warps (the aggregated atomics use all lanes);
    // each thread loads SPLIT_U entries before it files any of them
    const long long n = e1 - e0, nr = (n + 31) / 32 * 32;
    const long long step = (long long)SPLIT_U * blockDim.x;
    for (long long t0 = threadIdx.x; t0 < nr; t0 += step) {
        unsigned rsu[SPLIT_U];
#pragma unroll
        for (int u = 0; u < SPLIT_U; ++u) {
            const long long t = t0 + (long long)u * blockDim.x;
            rsu[u] = t < n ? (unsigned)brs[e0 + t] : 0u;
        }
#pragma unroll
        for (int u = 0; u < SPLIT_U; ++u) {
            const bool on = t0 + (long long)u * blockDim.x < n;
            const unsigned rs = rsu[u];
            const int br = (int)(rs >> 29), pr = (int)((rs >> 17) & 0xFFF);
            const int bs = (int)((rs >> 14) & 0x7), ps = (int)((rs >> 2) & 0xFFF);
            const int j1 = on ? job_of(jbb, jbd, tb.nblk, nj, br, pr) : -1;
            smem_agg_add(cnt, j1 >= 0 ? j1 : 0, j1 >= 0);
            const int j2 = on && !(rs & 1u) ? job_of(jbb, jbd, tb.nblk, nj, bs, ps) : -1;
            smem_agg_add(cnt, j2 >= 0 ? j2 : 0, j2 >= 0);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int j = 0; j < nj; ++j) {
            jstart[bb + j] = 2 * e0 + run;
            jcount[bb + j] = cnt[j];
            cur[j] = run;
            run += cnt[j];
        }
    }
    __syncthreads();
    for (long long t0 = threadIdx.x; t0 < nr; t0 += step) {
        unsigned rsu[SPLIT_U];
        double vu[SPLIT_U];
#pragma unroll
        for (int u = 0; u < SPLIT_U; ++u) {
            const long long t = t0 + (long long)u * blockDim.x;
            rsu[u] = t < n ? (unsigned)brs[e0 + t] : 0u;
            vu[u] = t < n ? bval[e0 + t] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < SPLIT_U; ++u) {
            const bool on = t0 + (long long)u * blockDim.x < n;
            const unsigned rs = rsu[u];
            const double v = vu[u];
            const int br = (int)(rs >> 29), pr = (int)((rs >> 17) & 0xFFF);
            const int bs = (int)((rs >> 14) & 0x7), ps = (int)((rs >> 2) & 0xFFF);
            const int j1 = on ? job_of(jbb, jbd, tb.nblk, nj, br, pr) : -1;
            const int s1 = smem_agg_add(cur, j1 >= 0 ? j1 : 0, j1 >= 0);
            if (j1 >= 0) {
                oval[2 * e0 + s1] = v;
                ors[2 * e0 + s1] = (pr << 16) | ps;
            }
            const int j2 = on && !(rs & 1u) ? job_of(jbb, jbd, tb.nblk, nj, bs, ps) : -1;
            const int s2 = smem_agg_add(cur, j2 >= 0 ? j2 : 0, j2 >= 0);
            if (j2 >= 0) {
                oval[2 * e0 + s2] = v;
                ors[2 * e0 + s2] = (ps << 16) | pr;
            }
        }
    }
}

// One CTA per (job, pq of the chunk): job = (GEMM1 group, band of r rows).
// The band of G_pq(r,s) is accumulated in shared memory from the bucket of
// (pq, job) -- exactly the elements of this band -- then written as GEMM1
// operand rows: FP64 [r][pql][nk] (nslices == 0) or BF16 digit slices
// [t][r*npc + pql][Kp] with row exponents (split path).
template <int NS>
__global__ void __launch_bounds__(256) k_expand_rows(const double* __restrict__ bval,
                                                     const int* __restrict__ brs,
                                                     const long long* __restrict__ jstart,
                                                     const int* __restrict__ jcount,
                                                     const ExpandJob* __restrict__ jobs,
                                                     long long bbase, int npc,
                                                     double* __restrict__ out_f64,
                                                     __nv_bfloat16* __restrict__ out_sl,
                                                     int* __restrict__ out_exp) {
    extern __shared__ double tile[];
    const ExpandJob J = jobs[blockIdx.x];
    const int pql = blockIdx.y;
    const int rows = J.r_hi - J.r_lo, nk = J.nk;
    for (int i = threadIdx.x; i < rows * nk; i += blockDim.x) tile[i] = 0.0;
    __syncthreads();
    const long long bk = bbase + (long long)pql * gridDim.x + blockIdx.x;
    const long long e0 = jstart[bk], ne = jcount[bk];
    // EXPAND_U entries per thread are loaded before any is added, so their
    // global loads overlap instead of one latency per entry
    for (long long b = threadIdx.x; b < ne; b += (long long)EXPAND_U * blockDim.x) {
        int rs[EXPAND_U];
        double v[EXPAND_U];
#pragma unroll
        for (int u = 0; u < EXPAND_U; ++u) {
            const long long i = b + (long long)u * blockDim.x;
            rs[u] = i < ne ? brs[e0 + i] : -1;
            v[u] = i < ne ? bval[e0 + i] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < EXPAND_U; ++u) {
            const int pr = (rs[u] >> 16) - J.r_lo, ps = rs[u] & 0xFFFF;
            if (rs[u] >= 0 && pr >= 0 && pr < rows && ps < nk) atomicAdd(&tile[pr * nk + ps], v[u]);
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (NS == 0) {
        double* o = out_f64 + J.out_pp * npc;
        for (int i = warp; i < rows; i += nw) {
            const long long rowo = ((long long)(J.r_lo + i) * npc + pql) * nk;
            for (int k = lane; k < nk; k += 32) o[rowo + k] = tile[i * nk + k];
        }
    } else {
        __nv_bfloat16* o = out_sl + J.out_pp * npc;
        const long long M = (long long)J.nr * npc;
        for (int i = warp; i < rows; i += nw) {
            const double* p = tile + i * nk;
            int S = -2000;
            const int wide = slicing_wide(nk);
            for (int k = lane; k < nk; k += 32) S = max(S, scale_exp_f64(p[k], wide));
            for (int q = 16; q; q >>= 1) S = max(S, __shfl_xor_sync(0xffffffffu, S, q));
            const long long row = (long long)(J.r_lo + i) * npc + pql;
            if (lane == 0) out_exp[J.exp_pp * npc + row] = S;
            const float sc = pow2f_safe(-S);
            for (int k0 = lane * 2; k0 < J.kp; k0 += 64) {
                __nv_bfloat16 d0[NS > 0 ? NS : 1], d1[NS > 0 ? NS : 1];
                float2 v0 = make_float2(0.f, 0.f), v1 = v0;
                if (S > -1000) {
                    if (k0 < nk) v0 = ff_from_double(p[k0]);
                    if (k0 + 1 < nk) v1 = ff_from_double(p[k0 + 1]);
                }
                ff_digits<NS>(v0.x * sc, v0.y * sc, d0);
                ff_digits<NS>(v1.x * sc, v1.y * sc, d1);
#pragma unroll
                for (int t = 0; t < NS; ++t) {
                    const uint32_t w = (uint32_t)__bfloat16_as_ushort(d0[t]) |
                                       ((uint32_t)__bfloat16_as_ushort(d1[t]) << 16);
                    *reinterpret_cast<uint32_t*>(o + ((long long)t * M + row) * J.kp + k0) = w;
                }
            }
        }
    }
}

void launch_bucket(cudaStream_t st, const double* rint, const int* l2, const int* l1, long long nint,
                   const long long* rec_off, const int2* rec_meta, int nrec, const ScatterTabs& tb,
                   int P, int* count, long long* off, double* bval, int* brs, long long nb,
                   long long* jstart, int* jcount, double* jval, int* jrs,
                   unsigned int* status) {
    cudaMemsetAsync(jcount, 0, sizeof(int) * (nb > 0 ? nb : 1), st);
    cudaMemsetAsync(count, 0, sizeof(int) * (P + 1), st);
    if (nint > 0) {
        long long blocks = (nint + 255) / 256;
        if (blocks > 152LL * 32) blocks = 152LL * 32;
        k_bucket_count<<<(unsigned)blocks, 256, 0, st>>>(rint, l2, l1, nint, rec_off, rec_meta,
                                                         nrec, tb, count, status);
    }
    k_scan_counts<<<1, 1024, 0, st>>>(count, P, off);
    cudaMemsetAsync(count, 0, sizeof(int) * (P + 1), st);
    if (nint > 0) {
        long long blocks = (nint + 255) / 256;
        if (blocks > 152LL * 32) blocks = 152LL * 32;
        k_bucket_place<<<(unsigned)blocks, 256, 0, st>>>(rint, l2, l1, nint, rec_off, rec_meta,
                                                         nrec, tb, off, count, bval, brs, status);
    }
    if (nint > 0)
        k_bucket_split<<<(unsigned)P, 256, 0, st>>>(off, bval, brs, tb, jstart, jcount, jval, jrs);
}

void raise_dyn_smem(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> set;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;  // the launch reports the error
    std::lock_guard<std::mutex> lk(mu);
    size_t& cur = set[{kernel, dev}];
    if (bytes <= cur) return;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess)
        cur = bytes;
}

void launch_expand_rows(cudaStream_t st, int nslices, const double* bval, const int* brs,
                        const long long* jstart, const int* jcount, const ExpandJob* jobs, int njobs,
                        long long bbase, int npc, size_t smem, double* out_f64,
                        __nv_bfloat16* out_sl, int* out_exp) {
    dim3 grid(njobs, npc);
#define RT_EXPAND(NSV)                                                                          \
    do {                                                                                        \
        raise_dyn_smem((const void*)k_expand_rows<NSV>, smem);                                  \
        k_expand_rows<NSV><<<grid, 256, smem, st>>>(bval, brs, jstart, jcount, jobs, bbase, npc, \
                                                    out_f64, out_sl, out_exp);                  \
    } while (0)
    switch (nslices) {
        case 0: RT_EXPAND(0); break;
        case 2: RT_EXPAND(2); break;
        case 3: RT_EXPAND(3); break;
        case 4: RT_EXPAND(4); break;
        case 5: RT_EXPAND(5); break;
        default: RT_EXPAND(6); break;
    }
#undef RT_EXPAND
}

// ===========================================================================
// adjoint: dE/dC of E = sum_{ijkl} Gamma_ijkl (ij|kl)
// ===========================================================================

// In-place pair-exchange symmetrisation, 32 x 32 tiles of the m^2 x m^2
// complex matrix; the block of tile pair (bi, bj), bi <= bj, owns both tiles.
__global__ void k_gamma_sym(double2* __restrict__ g, long long M2) {
    __shared__ double2 ta[32][33], tb[32][33];
    const long long bi = blockIdx.y, bj = blockIdx.x;
    if (bi > bj) return;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const long long ra = bi * 32 + r, ca = bj * 32 + tx;  // tile (bi, bj)
        const long long rb = bj * 32 + r, cb = bi * 32 + tx;  // tile (bj, bi)
        ta[r][tx] = (ra < M2 && ca < M2) ? g[ca * M2 + ra] : make_double2(0.0, 0.0);
        tb[r][tx] = (rb < M2 && cb < M2) ? g[cb * M2 + rb] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    // element (ra, ca) of tile a pairs with (ca, ra), held in tile b at [tx][r]
    for (int r = ty; r < 32; r += 8) {
        const long long ra = bi * 32 + r, ca = bj * 32 + tx;
        const long long rb = bj * 32 + r, cb = bi * 32 + tx;
        const double2 a = ta[r][tx], at = tb[tx][r];
        const double2 b = tb[r][tx], bt = ta[tx][r];
        if (ra < M2 && ca < M2) g[ca * M2 + ra] = make_double2(0.5 * (a.x + at.x), 0.5 * (a.y + at.y));
        if (bi != bj && rb < M2 && cb < M2)
            g[cb * M2 + rb] = make_double2(0.5 * (b.x + bt.x), 0.5 * (b.y + bt.y));
    }
}

__global__ void k_gamma_permute(const double2* __restrict__ in, const int* __restrict__ u, int m,
                                double2* __restrict__ out) {
    // block (j, k) of the output, looping over l, threads over i
    const long long mm = m;
    const int j = (int)(blockIdx.x % (unsigned)m), kk = (int)(blockIdx.x / (unsigned)m);
    for (int l = 0; l < m; ++l) {
        const long long src = (((long long)u[l] * mm + u[kk]) * mm + u[j]) * mm;
        const long long dst = (((long long)l * mm + kk) * mm + j) * mm;
        for (int i = threadIdx.x; i < m; i += blockDim.x) out[dst + i] = in[src + u[i]];
    }
}

void launch_gamma_permute(cudaStream_t st, const double* in, const int* u, int m, double* out) {
    const long long nb = (long long)m * m;
    if (nb > 0x7fffffffLL) throw_dim("adjoint: NSP too large");
    k_gamma_permute<<<(unsigned)nb, 128, 0, st>>>((const double2*)in, u, m, (double2*)out);
}

void launch_gamma_sym(cudaStream_t st, double* gamma, int m) {
    const long long M2 = (long long)m * m;
    const long long T = (M2 + 31) / 32;
    if (T > 65535) throw_dim("adjoint: NSP^2 above 2^21");
    dim3 grid((unsigned)T, (unsigned)T), block(32, 8);
    k_gamma_sym<<<grid, block, 0, st>>>((double2*)gamma, M2);
}

// Contraction operand of item it = i0 + ij (Kramers-unique pair u = (I,J)).
// relk: Gamma indices k + m l of the distinct ordered pairs r related to u
// (-1: none), relc: +-1 (value s_r H_u) or +-2 (s_r conj(H_u)).  With
// T_r(y,x) = Gs(x,y,r) + sigma_yx Gs(ybar,xbar,r):
//   Ghat_re(y,x) = sum_r s_r T_r(y,x),  Ghat_im(y,x) = i sum_r (+-) s_r T_r(y,x)
// (- for conjugated relatives), written real-ified as rows
// ((ij*2 + plane)*2 + ri)*m + y, columns ri_out*m + x:  [Re Im; -Im Re].
template <class E>
__global__ void k_gamma_hat(const double2* __restrict__ gs, int m, const int4* __restrict__ relk,
                            const int4* __restrict__ relc, const int* __restrict__ itrmo, int i0,
                            typename E::T* __restrict__ out) {
    const int ij = blockIdx.x, y = blockIdx.y;
    const int it = i0 + ij;
    const int4 rk = relk[it], rc = relc[it];
    const int kr[4] = {rk.x, rk.y, rk.z, rk.w}, cr[4] = {rc.x, rc.y, rc.z, rc.w};
    const int ty_ = itrmo[y];
    const int yb = abs(ty_) - 1;
    const long long M2 = (long long)m * m;
    const long long ldo = 2LL * m;
    for (int x = threadIdx.x; x < m; x += blockDim.x) {
        const int tx_ = itrmo[x];
        const int xb = abs(tx_) - 1;
        const double sg = ((ty_ > 0) == (tx_ > 0)) ? 1.0 : -1.0;
        double2 vr = make_double2(0.0, 0.0), vi = make_double2(0.0, 0.0);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (kr[r] < 0) continue;
            const long long base = (long long)kr[r] * M2;
            const double2 g1 = gs[base + x + (long long)m * y];
            const double2 g2 = gs[base + yb + (long long)m * xb];
            const double tr = g1.x + sg * g2.x, ti = g1.y + sg * g2.y;
            const double s = cr[r] > 0 ? 1.0 : -1.0;
            const double si = (cr[r] == 2 || cr[r] == -2) ? -s : s;
            vr.x += s * tr;
            vr.y += s * ti;
            vi.x -= si * ti;  // i * (tr + i ti) = -ti + i tr
            vi.y += si * tr;
        }
        const long long row0 = ((long long)ij * 2) * 2 * m + y;  // plane 0, ri 0
#pragma unroll
        for (int pl = 0; pl < 2; ++pl) {
            const double2 v = pl ? vi : vr;
            const long long ra = row0 + (long long)pl * 2 * m, rb = ra + m;
            out[ra * ldo + x] = E::from(v.x);
            out[ra * ldo + m + x] = E::from(v.y);
            out[rb * ldo + x] = E::from(-v.y);
            out[rb * ldo + m + x] = E::from(v.x);
        }
    }
}

void launch_gamma_hat(cudaStream_t st, bool ff, const double* gamma, int m, const int4* relk,
                      const int4* relc, const int* itrmo, int i0, int nij, double* out) {
    if (m > 65535) throw_dim("adjoint: NSP above 65535");
    dim3 grid((unsigned)nij, (unsigned)m);
    const int threads = m < 256 ? (m + 31) / 32 * 32 : 256;
    if (ff)
        k_gamma_hat<FFEl><<<grid, threads, 0, st>>>((const double2*)gamma, m, relk, relc, itrmo, i0,
                                                     (float2*)out);
    else
        k_gamma_hat<F64El><<<grid, threads, 0, st>>>((const double2*)gamma, m, relk, relc, itrmo, i0,
                                                      out);
}

// The same operand transposed, as float-float rows (ri_out*m + x) of length
// ldk over the K index ((ij*2 + plane)*2 + ri)*m + y (the K-major layout
// the tensor-core path slices); one block per (ij, x), threads over y.
__global__ void k_gamma_hat_t(const double2* __restrict__ gs, int m, const int4* __restrict__ relk,
                              const int4* __restrict__ relc, const int* __restrict__ itrmo, int i0,
                              long long ldk, float2* __restrict__ out) {
    const int ij = blockIdx.x, x = blockIdx.y;
    const int it = i0 + ij;
    const int4 rk = relk[it], rc = relc[it];
    const int kr[4] = {rk.x, rk.y, rk.z, rk.w}, cr[4] = {rc.x, rc.y, rc.z, rc.w};
    const int tx_ = itrmo[x];
    const int xb = abs(tx_) - 1;
    const long long M2 = (long long)m * m;
    for (int y = threadIdx.x; y < m; y += blockDim.x) {
        const int ty_ = itrmo[y];
        const int yb = abs(ty_) - 1;
        const double sg = ((ty_ > 0) == (tx_ > 0)) ? 1.0 : -1.0;
        double2 vr = make_double2(0.0, 0.0), vi = make_double2(0.0, 0.0);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            if (kr[r] < 0) continue;
            const long long base = (long long)kr[r] * M2;
            const double2 g1 = gs[base + x + (long long)m * y];
            const double2 g2 = gs[base + yb + (long long)m * xb];
            const double tr = g1.x + sg * g2.x, ti = g1.y + sg * g2.y;
            const double s = cr[r] > 0 ? 1.0 : -1.0;
            const double si = (cr[r] == 2 || cr[r] == -2) ? -s : s;
            vr.x += s * tr;
            vr.y += s * ti;
            vi.x -= si * ti;
            vi.y += si * tr;
        }
#pragma unroll
        for (int pl = 0; pl < 2; ++pl) {
            const double2 v = pl ? vi : vr;
            const long long ka = ((long long)(ij * 2 + pl) * 2) * m + y, kb = ka + m;
            out[(long long)x * ldk + ka] = FFEl::from(v.x);        // (ri 0, re out)
            out[(long long)(m + x) * ldk + ka] = FFEl::from(v.y);  // (ri 0, im out)
            out[(long long)x * ldk + kb] = FFEl::from(-v.y);       // (ri 1, re out)
            out[(long long)(m + x) * ldk + kb] = FFEl::from(v.x);  // (ri 1, im out)
        }
    }
}

void launch_gamma_hat_t(cudaStream_t st, const double* gamma, int m, const int4* relk,
                        const int4* relc, const int* itrmo, int i0, int nij, long long ldk,
                        double* out) {
    if (m > 65535) throw_dim("adjoint: NSP above 65535");
    dim3 grid((unsigned)nij, (unsigned)m);
    const int threads = m < 256 ? (m + 31) / 32 * 32 : 256;
    k_gamma_hat_t<<<grid, threads, 0, st>>>((const double2*)gamma, m, relk, relc, itrmo, i0, ldk,
                                            (float2*)out);
}

// Fixed-order sum of split-K partial products into the FP64 accumulator.
template <class E>
__global__ void k_partial_sum(const typename E::T* __restrict__ part, int nb, long long len,
                              double* __restrict__ acc) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < len;
         i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nb; ++b) s += E::val(part[(long long)b * len + i]);
        acc[i] += s;
    }
}

void launch_partial_sum(cudaStream_t st, bool ff, const double* part, int nb, long long len,
                        double* acc) {
    const unsigned g = (unsigned)std::min<long long>((len + 255) / 256, 152LL * 8);
    if (ff)
        k_partial_sum<FFEl><<<g, 256, 0, st>>>((const float2*)part, nb, len, acc);
    else
        k_partial_sum<F64El><<<g, 256, 0, st>>>(part, nb, len, acc);
}

}  // namespace rt
