// rt_fock.cu -- tmoone's skeleton Fock build on the GPU (replaces MFDFOCK,
// source/tmoone/mfdfock.F:53-140, and FOCK, source/tmoone/fock.F:1-656).
//
// Every unique integral (IJ|KL) of a record of type IT (the index-coincidence
// type of INTTYP) adds products "integral x density element x small factor"
// to lower-triangle Fock elements T(x,y) = x(x-1)/2 + y of the four arrays
// AAR, BAR, AAI, BAI, in up to two density sets (closed and open shell).
// FOCK spells the fourteen types out one by one; here each type is a short
// table of terms -- target pair, source pair (positions in (I,J,K,L)) and one
// integer factor per array -- read from constant memory:
//
//   F_x(target) += (integral * D_x(source)) * factor_x      x = AAR..BAI
//
// The integrals stay where the transform keeps them (HBM, 16 bytes each);
// a persistent grid walks the records in chunks of up to 4096 integrals, one
// chunk per block at a time (a record has one type, so the term table is
// uniform across the block).  The additions are FP64 atomics into
// the Fock arrays (a few MB, resident in L2).  Where a whole warp adds to
// the same element -- records list many integrals of one (I,J) pair in a
// row -- the warp sums its contributions first and adds once.
#include <cuda_runtime.h>

#include <cstdint>

#include "rt_kernels.h"

namespace rt {

namespace {

struct FockTerm {
    int8_t tx, ty, sx, sy;  // target pair and source pair, positions 0..3 of (I,J,K,L)
    int8_t c[4];            // factor per array: AAR, BAR, AAI, BAI
};
struct FockType {
    int nterm;
    FockTerm t[6];
};

// I = 0, J = 1, K = 2, L = 3; the fock.F lines each row restates
#define FT_(tx, ty, sx, sy, a, b, c, d) {tx, ty, sx, sy, {a, b, c, d}}
#define FT(...) FT_(__VA_ARGS__)
#define ALL(v) v, v, v, v
__constant__ FockType c_fock_types[15] = {
    {0, {}},
    // 1 (fock.F:52-65): (II|II)
    {1, {FT(0, 1, 0, 1, 1, -1, -1, -1)}},
    // 2 (fock.F:72-107)
    {3, {FT(0, 1, 0, 1, 3, 1, 1, 1), FT(1, 3, 0, 2, ALL(-1)), FT(0, 2, 1, 3, ALL(-1))}},
    // 3 (fock.F:115-138)
    {3, {FT(0, 1, 2, 3, 2, 0, 0, 0), FT(2, 3, 0, 1, 2, 0, 0, 0), FT(0, 2, 0, 2, ALL(-1))}},
    // 4 (fock.F:146-164)
    {2, {FT(0, 1, 2, 3, 2, 0, 0, 0), FT(2, 3, 0, 1, 1, -1, -1, -1)}},
    // 5 (fock.F:172-206)
    {4, {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 2, 0, 0, 0), FT(0, 3, 1, 2, ALL(-1)),
         FT(1, 2, 0, 3, ALL(-1))}},
    // 6 (fock.F:214-232)
    {2, {FT(2, 3, 0, 1, 2, 0, 0, 0), FT(0, 1, 2, 3, 1, -1, -1, -1)}},
    // 7 (fock.F:240-274)
    {4, {FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 1, 2, 3, 2, 0, 0, 0), FT(0, 2, 1, 3, ALL(-1)),
         FT(1, 3, 0, 2, ALL(-1))}},
    // 8 (fock.F:282-316)
    {4, {FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 1, 2, 3, 2, 0, 0, 0), FT(0, 2, 3, 1, -1, 1, 1, 1),
         FT(3, 1, 0, 2, -1, 1, 1, 1)}},
    // 9 (fock.F:324-364)
    {4, {FT(0, 1, 2, 3, 3, -1, -1, -1), FT(2, 3, 0, 1, 3, -1, -1, -1), FT(0, 3, 1, 2, -1, -1, 1, -1),
         FT(1, 2, 0, 3, -2, 0, 0, 0)}},
    // 10 (fock.F:372-412)
    {4, {FT(0, 1, 2, 3, 3, 1, 1, 1), FT(2, 3, 0, 1, 3, 1, 1, 1), FT(0, 2, 1, 3, -2, 0, 0, 0),
         FT(1, 3, 0, 2, ALL(-1))}},
    // 11 (fock.F:420-460)
    {4, {FT(0, 1, 2, 3, 3, 1, 1, 1), FT(2, 3, 0, 1, 3, 1, 1, 1), FT(0, 2, 1, 3, ALL(-1)),
         FT(1, 3, 0, 2, -2, 0, 0, 0)}},
    // 12 (fock.F:468-522)
    {6, {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 3, 1, 2, ALL(-1)),
         FT(1, 2, 0, 3, ALL(-1)), FT(0, 2, 1, 3, ALL(-1)), FT(1, 3, 0, 2, ALL(-1))}},
    // 13 (fock.F:530-584)
    {6, {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 3, 2, 1, -1, 1, 1, 1),
         FT(2, 1, 0, 3, -1, 1, 1, 1), FT(0, 2, 1, 3, ALL(-1)), FT(1, 3, 0, 2, ALL(-1))}},
    // 14 (fock.F:593-647)
    {6, {FT(0, 1, 2, 3, 4, 0, 0, 0), FT(2, 3, 0, 1, 4, 0, 0, 0), FT(0, 3, 2, 1, -1, 1, 1, 1),
         FT(2, 1, 0, 3, -1, 1, 1, 1), FT(0, 2, 3, 1, -1, 1, 1, 1), FT(3, 1, 0, 2, -1, 1, 1, 1)}},
};
#undef ALL
#undef FT
#undef FT_

__device__ __forceinline__ int pick(int i, int j, int k, int l, int pos) {
    return pos == 0 ? i : pos == 1 ? j : pos == 2 ? k : l;
}

__device__ __forceinline__ long long tri0(int x, int y) { return (long long)x * (x - 1) / 2 + y - 1; }

__global__ void __launch_bounds__(256) k_fock_skeleton(const double* __restrict__ rint,
                                                       const int* __restrict__ l2,
                                                       const int* __restrict__ l1,
                                                       const FockRec* __restrict__ recs, int nrec,
                                                       int nsc, long long ntri, int nmat,
                                                       const double* __restrict__ dens,
                                                       double* __restrict__ fock,
                                                       unsigned long long* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    for (int r = blockIdx.x; r < nrec; r += gridDim.x) {
        const FockRec R = recs[r];
        const FockType& T = c_fock_types[R.it];
        for (long long base = 0; base < R.nt; base += blockDim.x) {
            const long long t = base + threadIdx.x;
            bool on = t < R.nt;
            int i = 1, j = 1, k = 1, l = 1;
            double v = 0.0;
            if (on) {
                const unsigned u2 = (unsigned)l2[R.off + t], u1 = (unsigned)l1[R.off + t];
                i = (int)(u2 >> 16), j = (int)(u2 & 0xFFFFu), k = (int)(u1 >> 16), l = (int)(u1 & 0xFFFFu);
                if (i < 1 || i > nsc || j < 1 || j > nsc || k < 1 || k > nsc || l < 1 || l > nsc) {
                    atomicOr(bad, 1ull);
                    on = false;
                    i = j = k = l = 1;
                } else {
                    v = rint[R.off + t];
                }
            }
            const unsigned on_mask = __ballot_sync(0xffffffffu, on);
            if (on_mask == 0) continue;
            const int leader = __ffs(on_mask) - 1;
            for (int q = 0; q < T.nterm; ++q) {
                const FockTerm m = T.t[q];
                const long long tg = tri0(pick(i, j, k, l, m.tx), pick(i, j, k, l, m.ty));
                const long long sr = tri0(pick(i, j, k, l, m.sx), pick(i, j, k, l, m.sy));
                const long long tg0 = __shfl_sync(0xffffffffu, tg, leader);
                const bool uniform = __all_sync(0xffffffffu, !on || tg == tg0);
                for (int s = 0; s < nmat; ++s) {
                    const double* d = dens + (long long)s * 4 * ntri;
                    double* f = fock + (long long)s * 4 * ntri;
#pragma unroll
                    for (int x = 0; x < 4; ++x) {
                        if (m.c[x] == 0) continue;
                        double c = on ? (v * d[x * ntri + sr]) * (double)m.c[x] : 0.0;
                        if (uniform) {
#pragma unroll
                            for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
                            if (lane == leader) atomicAdd(f + x * ntri + tg0, c);
                        } else if (on) {
                            atomicAdd(f + x * ntri + tg, c);
                        }
                    }
                }
            }
        }
    }
}

}  // namespace

void launch_fock_skeleton(cudaStream_t st, const double* rint, const int* l2, const int* l1,
                          const FockRec* recs, int nrec, int nsc, int nmat, const double* dens,
                          double* fock, unsigned long long* bad) {
    if (nrec <= 0) return;
    const long long ntri = (long long)nsc * (nsc + 1) / 2;
    const int grid = nrec < 152 * 8 ? nrec : 152 * 8;
    k_fock_skeleton<<<grid, 256, 0, st>>>(rint, l2, l1, recs, nrec, nsc, ntri, nmat, dens, fock, bad);
}

}  // namespace rt
