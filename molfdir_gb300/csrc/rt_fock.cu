// rt_fock.cu -- tmoone's skeleton Fock build on the GPU (replaces MFDFOCK,
// source/tmoone/mfdfock.F:53-140, with FOCK, source/tmoone/fock.F:1-656,
// and MFDBREIT, source/tmoone/mfdbreit.F:50-138, with GAUNT,
// source/tmoone/gaunt.F).
//
// Every unique integral (IJ|KL) of a record of type IT (the index-coincidence
// type of INTTYP) adds products "integral x density element x small factor"
// to lower-triangle Fock elements T(x,y) = x(x-1)/2 + y of the four arrays
// AAR, BAR, AAI, BAI, in up to two density sets (closed and open shell).
// FOCK spells the fourteen types out one by one; here each type is a short
// table of terms -- target pair, source pair (positions in (I,J,K,L)) and one
// integer factor per array:
//
//   F_x(target) += (integral * D_x(source)) * factor_x      x = AAR..BAI
//
// The integrals stay where the transform keeps them (HBM, 16 bytes each);
// a persistent grid walks the records in chunks of up to 4096 integrals, one
// chunk per block at a time (a record has one type, so the term table is
// uniform across the block).  The additions are FP64 atomics into
// the Fock arrays (a few MB, resident in L2).  The term lists are expanded at
// compile time per type (the kernel is bound by instruction issue, not by
// the atomics).  Where a whole warp adds to the same element -- records list
// many integrals of one label pair in a row -- the warp sums first and adds
// once.
#include <cuda_runtime.h>

#include <cstdint>

#include "rt_kernels.h"

namespace rt {

namespace {

struct FockTerm {
    int tx, ty, sx, sy;  // target pair and source pair, positions 0..3 of (I,J,K,L)
    int c[4];            // factor per array: AAR, BAR, AAI, BAI
};

// The terms of type `it` (1..14), I = 0, J = 1, K = 2, L = 3, with the
// fock.F lines each row restates; evaluated at compile time.
__host__ __device__ constexpr int fock_nterm(int it) {
    return it == 1 ? 1 : it == 2 || it == 3 ? 3 : it == 4 || it == 6 ? 2 : it >= 12 ? 6 : 4;
}
__host__ __device__ constexpr FockTerm fock_term(int it, int q) {
#define FT_(tx, ty, sx, sy, a, b, c, d) FockTerm{tx, ty, sx, sy, {a, b, c, d}}
#define FT(...) FT_(__VA_ARGS__)
#define ALL(v) v, v, v, v
    const FockTerm t[15][6] = {
        {},
        // 1 (fock.F:52-65)
        {FT(0, 1, 0, 1, 1, -1, -1, -1)},
        // 2 (fock.F:72-107)
        {FT(0, 1, 0, 1, 3, 1, 1, 1), FT(1, 3, 0, 2, ALL(-1)), FT(0, 2, 1, 3, ALL(-1))},
        // 3 (fock.F:115-138)
        {FT(0, 1, 2, 3, 2, 0, 0, 0), FT(2, 3, 0, 1, 2, 0, 0, 0), FT(0, 2, 0, 2, ALL(-1))},
        // 4 (fock.F:146-164)
        {FT(0, 1, 2, 3, 2, 0, 0, 0), FT(2, 3, 0, 1, 1, -1, -1, -1)},
        // 5 (fock.F:172-206)
        {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 2, 0, 0, 0), FT(0, 3, 1, 2, ALL(-1)),
         FT(1, 2, 0, 3, ALL(-1))},
        // 6 (fock.F:214-232)
        {FT(2, 3, 0, 1, 2, 0, 0, 0), FT(0, 1, 2, 3, 1, -1, -1, -1)},
        // 7 (fock.F:240-274)
        {FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 1, 2, 3, 2, 0, 0, 0), FT(0, 2, 1, 3, ALL(-1)),
         FT(1, 3, 0, 2, ALL(-1))},
        // 8 (fock.F:282-316)
        {FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 1, 2, 3, 2, 0, 0, 0), FT(0, 2, 3, 1, -1, 1, 1, 1),
         FT(3, 1, 0, 2, -1, 1, 1, 1)},
        // 9 (fock.F:324-364)
        {FT(0, 1, 2, 3, 3, -1, -1, -1), FT(2, 3, 0, 1, 3, -1, -1, -1), FT(0, 3, 1, 2, -1, -1, 1, -1),
         FT(1, 2, 0, 3, -2, 0, 0, 0)},
        // 10 (fock.F:372-412)
        {FT(0, 1, 2, 3, 3, 1, 1, 1), FT(2, 3, 0, 1, 3, 1, 1, 1), FT(0, 2, 1, 3, -2, 0, 0, 0),
         FT(1, 3, 0, 2, ALL(-1))},
        // 11 (fock.F:420-460)
        {FT(0, 1, 2, 3, 3, 1, 1, 1), FT(2, 3, 0, 1, 3, 1, 1, 1), FT(0, 2, 1, 3, ALL(-1)),
         FT(1, 3, 0, 2, -2, 0, 0, 0)},
        // 12 (fock.F:468-522)
        {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 3, 1, 2, ALL(-1)),
         FT(1, 2, 0, 3, ALL(-1)), FT(0, 2, 1, 3, ALL(-1)), FT(1, 3, 0, 2, ALL(-1))},
        // 13 (fock.F:530-584)
        {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 3, 2, 1, -1, 1, 1, 1),
         FT(2, 1, 0, 3, -1, 1, 1, 1), FT(0, 2, 1, 3, ALL(-1)), FT(1, 3, 0, 2, ALL(-1))},
        // 14 (fock.F:593-647)
        {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 3, 2, 1, -1, 1, 1, 1),
         FT(2, 1, 0, 3, -1, 1, 1, 1), FT(0, 2, 3, 1, -1, 1, 1, 1), FT(3, 1, 0, 2, -1, 1, 1, 1)},
    };
#undef ALL
#undef FT
#undef FT_
    return t[it][q];
}

// The terms of tmoone's GAUNT (source/tmoone/gaunt.F) for the types it
// accepts (2, 10, 11, 13, 14; the others stop it with Q2JOB class 6,
// gaunt.F:25-28, and are refused on the host).
__host__ __device__ constexpr int gaunt_nterm(int it) { return it == 2 ? 3 : 4; }
__host__ __device__ constexpr FockTerm gaunt_term(int it, int q) {
#define FT_(tx, ty, sx, sy, a, b, c, d) FockTerm{tx, ty, sx, sy, {a, b, c, d}}
#define FT(...) FT_(__VA_ARGS__)
    const FockTerm t2[3] = {  // gaunt.F:41-76, I = K > J = L
        FT(0, 1, 0, 1, 3, 1, 1, 1), FT(1, 3, 0, 2, 3, -1, -1, -1), FT(0, 2, 1, 3, 3, -1, -1, -1)};
    const FockTerm t10[4] = {  // gaunt.F:84-124, I = K > J > L
        FT(0, 1, 2, 3, 3, 1, 1, 1), FT(2, 3, 0, 1, 3, 1, 1, 1), FT(0, 2, 1, 3, 6, 0, 0, 0),
        FT(1, 3, 0, 2, 3, 1, -1, 1)};
    const FockTerm t11[4] = {  // gaunt.F:132-172, I > K > J = L
        FT(0, 1, 2, 3, 3, 1, 1, 1), FT(2, 3, 0, 1, 3, 1, 1, 1), FT(0, 2, 1, 3, 3, -1, -1, -1),
        FT(1, 3, 0, 2, 6, 0, 0, 0)};
    const FockTerm t13[4] = {  // gaunt.F:180-228, I > K > J > L
        FT(0, 3, 2, 1, 3, 1, 1, 1), FT(2, 1, 0, 3, 3, 1, 1, 1), FT(0, 2, 1, 3, 3, -1, -1, -1),
        FT(1, 3, 0, 2, 3, -1, -1, -1)};
    const FockTerm t14[4] = {  // gaunt.F:236-284, I > K > L > J
        FT(0, 3, 2, 1, 3, 1, 1, 1), FT(2, 1, 0, 3, 3, 1, 1, 1), FT(0, 2, 3, 1, 3, 1, 1, 1),
        FT(3, 1, 0, 2, 3, 1, 1, 1)};
#undef FT
#undef FT_
    return it == 2 ? t2[q] : it == 10 ? t10[q] : it == 11 ? t11[q] : it == 13 ? t13[q] : t14[q];
}

template <bool G>
__host__ __device__ constexpr int nterm_of(int it) { return G ? gaunt_nterm(it) : fock_nterm(it); }
template <bool G>
__host__ __device__ constexpr FockTerm term_of(int it, int q) { return G ? gaunt_term(it, q) : fock_term(it, q); }

template <int P>
__device__ __forceinline__ unsigned pick(unsigned i, unsigned j, unsigned k, unsigned l) {
    if constexpr (P == 0) return i;
    else if constexpr (P == 1) return j;
    else if constexpr (P == 2) return k;
    else return l;
}

// 0-based lower-triangle position x(x-1)/2 + y - 1 (fits 32 bits for x, y <= 65535)
__device__ __forceinline__ unsigned tri0(unsigned x, unsigned y) { return x * (x - 1) / 2 + y - 1; }

// Products in the integer units.  GB300 issues FP64 arithmetic at a small
// fraction of its integer rate, and each term and array needs one product
// integral x density element, so the products are formed from the binary64
// fields directly: the 53-bit significands multiplied into the high 64 bits
// of their 106-bit product (one 64x64 high multiply), renormalised by one
// bit where the product is 2 or more, rounded to nearest on the first
// dropped bit, and given the summed exponent plus log2 of the term's
// power-of-two factor.  The result is within one unit in the last place of
// the exact product (the discarded low 64 bits only decide ties), which the
// tolerance of the sums (1e-12 of the largest element) does not see.  Zero
// and subnormal operands give zero; the integrals and densities are normal
// numbers far from overflow.
__device__ __forceinline__ double mul_pow2(double a, double b, int log2f, unsigned long long flip) {
    const unsigned long long ua = (unsigned long long)__double_as_longlong(a);
    const unsigned long long ub = (unsigned long long)__double_as_longlong(b);
    const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
    if (ea == 0 || eb == 0) return 0.0;
    constexpr unsigned long long MANT = (1ull << 52) - 1, HIDDEN = 1ull << 52;
    const unsigned long long hi = __umul64hi(((ua & MANT) | HIDDEN) << 11, ((ub & MANT) | HIDDEN) << 11);
    const int two = (int)(hi >> 63);           // product of the significands >= 2
    const int sh = 10 + two;
    unsigned long long m = (hi >> sh) + ((hi >> (sh - 1)) & 1ull);
    int e = ea + eb - 1023 + two + log2f;
    if (m >> 53) {                             // rounding carried into bit 53
        m >>= 1;
        ++e;
    }
    if (e <= 0) return 0.0;
    const unsigned long long sign = ((ua ^ ub) & (1ull << 63)) ^ flip;
    return __longlong_as_double((long long)(sign | ((unsigned long long)e << 52) | (m & MANT)));
}

// The integral's multiple 3v (one FP64 multiply, made only for the types
// that use it); the factors 1, 2, 4 and the 2 of 6 enter through the exponent.
struct Multiples {
    double v1, v3;
};
// (C v) * dv for a term factor C in {1, 2, 3, 4, 6} up to sign
template <int C>
__device__ __forceinline__ double times(const Multiples& w, double dv) {
    constexpr int a = C < 0 ? -C : C;
    static_assert(a == 1 || a == 2 || a == 3 || a == 4 || a == 6, "term factor");
    constexpr unsigned long long flip = C < 0 ? (1ull << 63) : 0ull;
    if constexpr (a == 3 || a == 6) return mul_pow2(w.v3, dv, a == 6 ? 1 : 0, flip);
    else return mul_pow2(w.v1, dv, a == 1 ? 0 : a == 2 ? 1 : 2, flip);
}

// Term Q onwards of type IT for one integral per lane (lanes with on = false
// add nothing but take part in the warp votes).  When the whole warp adds to
// one element, one lane adds the warp's sum.
// F_x(tg) += (C v) D_x(sr) for array x of one density set
template <int C>
__device__ __forceinline__ void add_term(int x, bool on, bool uniform, int lane, int leader, const Multiples& w,
                                         const double* __restrict__ d, double* __restrict__ f, unsigned ntri,
                                         unsigned sr, unsigned tg, unsigned tg0) {
    if constexpr (C != 0) {
        double c = on ? times<C>(w, d[(size_t)x * ntri + sr]) : 0.0;
        if (uniform) {
#pragma unroll
            for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
            if (lane == leader) atomicAdd(f + (size_t)x * ntri + tg0, c);
        } else if (on) {
            atomicAdd(f + (size_t)x * ntri + tg, c);
        }
    }
}

template <bool G, int NM, int IT, int Q>
__device__ __forceinline__ void fock_terms(bool on, unsigned i, unsigned j, unsigned k, unsigned l,
                                           const Multiples& w, int lane, int leader, unsigned ntri,
                                           const double* __restrict__ dens, double* __restrict__ fock) {
    if constexpr (Q < nterm_of<G>(IT)) {
        constexpr FockTerm m = term_of<G>(IT, Q);
        const unsigned tg = tri0(pick<m.tx>(i, j, k, l), pick<m.ty>(i, j, k, l));
        const unsigned sr = tri0(pick<m.sx>(i, j, k, l), pick<m.sy>(i, j, k, l));
        const unsigned tg0 = __shfl_sync(0xffffffffu, tg, leader);
        const bool uniform = __all_sync(0xffffffffu, !on || tg == tg0);
#pragma unroll
        for (int s = 0; s < NM; ++s) {
            const double* d = dens + (size_t)s * 4 * ntri;
            double* f = fock + (size_t)s * 4 * ntri;
            add_term<m.c[0]>(0, on, uniform, lane, leader, w, d, f, ntri, sr, tg, tg0);
            add_term<m.c[1]>(1, on, uniform, lane, leader, w, d, f, ntri, sr, tg, tg0);
            add_term<m.c[2]>(2, on, uniform, lane, leader, w, d, f, ntri, sr, tg, tg0);
            add_term<m.c[3]>(3, on, uniform, lane, leader, w, d, f, ntri, sr, tg, tg0);
        }
        fock_terms<G, NM, IT, Q + 1>(on, i, j, k, l, w, lane, leader, ntri, dens, fock);
    }
}

// the integrals of one record chunk, all of type IT (G: GAUNT's terms)
template <bool G, int NM, int IT>
__device__ __forceinline__ void fock_chunk(const FockRec& R, const double* __restrict__ rint,
                                           const int* __restrict__ l2, const int* __restrict__ l1,
                                           unsigned nsc, unsigned ntri,
                                           const double* __restrict__ dens, double* __restrict__ fock,
                                           unsigned long long* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    for (long long base = 0; base < R.nt; base += blockDim.x) {
        const long long t = base + threadIdx.x;
        bool on = t < R.nt;
        unsigned i = 1, j = 1, k = 1, l = 1;
        double v = 0.0;
        if (on) {
            const unsigned u2 = (unsigned)l2[R.off + t], u1 = (unsigned)l1[R.off + t];
            i = u2 >> 16, j = u2 & 0xFFFFu, k = u1 >> 16, l = u1 & 0xFFFFu;
            if (i - 1 >= nsc || j - 1 >= nsc || k - 1 >= nsc || l - 1 >= nsc) {  // outside 1..nsc
                atomicOr(bad, 1ull);
                on = false;
                i = j = k = l = 1;
            } else {
                v = rint[R.off + t];
            }
        }
        const unsigned on_mask = __ballot_sync(0xffffffffu, on);
        if (on_mask == 0) continue;
        const Multiples w{v, 3.0 * v};   // 3v is made only where a type uses it
        fock_terms<G, NM, IT, 0>(on, i, j, k, l, w, lane, __ffs(on_mask) - 1, ntri, dens, fock);
    }
}

template <bool G, int NM>
__global__ void __launch_bounds__(256) k_fock_skeleton(const double* __restrict__ rint,
                                                       const int* __restrict__ l2,
                                                       const int* __restrict__ l1,
                                                       const FockRec* __restrict__ recs, int nrec,
                                                       unsigned nsc, unsigned ntri,
                                                       const double* __restrict__ dens,
                                                       double* __restrict__ fock,
                                                       unsigned long long* __restrict__ bad) {
    for (int r = blockIdx.x; r < nrec; r += gridDim.x) {
        const FockRec R = recs[r];
#define RT_FOCK_CASE(T) \
    case T: fock_chunk<G, NM, T>(R, rint, l2, l1, nsc, ntri, dens, fock, bad); break;
        if constexpr (G) {
            switch (R.it) {  // uniform across the block
                RT_FOCK_CASE(2) RT_FOCK_CASE(10) RT_FOCK_CASE(11) RT_FOCK_CASE(13) RT_FOCK_CASE(14)
                default: break;
            }
        } else {
            switch (R.it) {
                RT_FOCK_CASE(1) RT_FOCK_CASE(2) RT_FOCK_CASE(3) RT_FOCK_CASE(4) RT_FOCK_CASE(5)
                RT_FOCK_CASE(6) RT_FOCK_CASE(7) RT_FOCK_CASE(8) RT_FOCK_CASE(9) RT_FOCK_CASE(10)
                RT_FOCK_CASE(11) RT_FOCK_CASE(12) RT_FOCK_CASE(13) RT_FOCK_CASE(14)
                default: break;
            }
        }
#undef RT_FOCK_CASE
    }
}

}  // namespace

void launch_fock_skeleton(cudaStream_t st, bool gaunt, const double* rint, const int* l2, const int* l1,
                          const FockRec* recs, int nrec, int nsc, int nmat, const double* dens,
                          double* fock, unsigned long long* bad) {
    if (nrec <= 0) return;
    const unsigned ntri = (unsigned)((long long)nsc * (nsc + 1) / 2);
    // four blocks per SM, as many as are resident at 256 threads and the
    // two-set kernels' registers: a second wave would leave SMs idle at the
    // end, and more blocks per SM (the one-set kernels would fit eight)
    // measured slower
    const int grid = nrec < 152 * 4 ? nrec : 152 * 4;
#define RT_FOCK_LAUNCH(GV, NMV)                                                                          \
    k_fock_skeleton<GV, NMV><<<grid, 256, 0, st>>>(rint, l2, l1, recs, nrec, (unsigned)nsc, ntri, dens, fock, bad)
    if (gaunt) {
        if (nmat == 2) RT_FOCK_LAUNCH(true, 2);
        else RT_FOCK_LAUNCH(true, 1);
    } else {
        if (nmat == 2) RT_FOCK_LAUNCH(false, 2);
        else RT_FOCK_LAUNCH(false, 1);
    }
#undef RT_FOCK_LAUNCH
}

}  // namespace rt
