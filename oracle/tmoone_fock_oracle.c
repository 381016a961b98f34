/*
 * tmoone_fock_oracle.c -- CPU restatement of tmoone's skeleton Fock build
 * (MFDFOCK with FOCK).  TEST INFRASTRUCTURE ONLY: the parity oracle for the
 * GPU library's rt_fock_skeleton and its timed CPU baseline; no product code
 * path links or calls it.
 *
 * Parity status: "parity unpinned" against reference-run outputs (Fortran 77,
 * no compiler here, no tmoone fixtures in the reference).  The restatement is
 * cross-checked against dense formulations of the same integrals
 * (tests/test_fock_oracle.py): FOCK against 2J - K / -K, GAUNT against
 * 3K / -K for Kramers-restricted densities.
 *
 * MFDFOCK (source/tmoone/mfdfock.F:53-66) clears the closed- and open-shell
 * Fock arrays, then reads the integral records of files 1..MFIL
 * (mfdfock.F:68-140), unpacks each label pair (mfdfock.F:103-114: I, J from
 * the first label array, K, L from the second, 32-bit layout) and hands the
 * record to FOCK once per density set (mfdfock.F:121-127).  FOCK
 * (source/tmoone/fock.F) jumps on the record's integral type IT
 * (fock.F:37-38) and adds, per integral in record order, the products of the
 * integral with density elements to Fock elements, both addressed as lower
 * triangles T(x,y) = x(x-1)/2 + y.  The density and Fock sets are four
 * arrays each, in COMMON order AAR, BAR, AAI, BAI (densfock.inc:4-7); the
 * arithmetic below keeps the Fortran's operand order in each product.
 */
#include <stddef.h>

#include "rotran_oracle.h"

static inline long tri(long x, long y) { return x * (x - 1) / 2 + y - 1; }  /* 0-based */

/* One integral of type it with labels (i,j,k,l) and value r; d and f are
 * the four arrays AAR, BAR, AAI, BAI of n elements each, f += terms. */
static void fock_one(int it, long i, long j, long k, long l, double r, const double* d, double* f,
                     long n) {
    const double *daar = d, *dbar = d + n, *daai = d + 2 * n, *dbai = d + 3 * n;
    double *faar = f, *fbar = f + n, *faai = f + 2 * n, *fbai = f + 3 * n;
    const long ij = tri(i, j), kl = tri(k, l);
    long a, b;
    double c1, c2, c3, c4;
    switch (it) {
    case 1: /* fock.F:52-65 */
        faar[ij] += r * daar[ij];
        faai[ij] += -r * daai[ij];
        fbar[ij] += -r * dbar[ij];
        fbai[ij] += -r * dbai[ij];
        break;
    case 2: /* fock.F:72-107 */
        a = tri(i, k);
        b = tri(j, l);
        faar[ij] += 3.0 * r * daar[ij];
        faai[ij] += r * daai[ij];
        fbar[ij] += r * dbar[ij];
        fbai[ij] += r * dbai[ij];
        c1 = -r * daar[a], c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
        faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        c1 = -r * daar[b], c2 = -r * daai[b], c3 = -r * dbar[b], c4 = -r * dbai[b];
        faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
        break;
    case 3: /* fock.F:115-138 */
        a = tri(i, k);
        faar[ij] += r * 2.0 * daar[kl];
        faar[kl] += r * 2.0 * daar[ij];
        c1 = -r * daar[a], c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
        faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
        break;
    case 4: /* fock.F:146-164 */
    case 6: /* fock.F:214-232: the same two products with the pairs exchanged */
        a = it == 4 ? ij : kl;  /* pair whose density feeds the second term */
        b = it == 4 ? kl : ij;  /* pair that receives it */
        if (it == 4) faar[ij] += r * 2.0 * daar[kl];
        else faar[kl] += r * daar[ij] * 2.0;
        c3 = -r * dbar[a];  /* FCABR */
        c4 = r * dbai[a];   /* FCABI */
        c1 = r * daar[a];
        c2 = -r * daai[a];
        faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] -= c4;
        break;
    case 5: /* fock.F:172-206 */
    case 7: /* fock.F:240-274 */
    case 12: /* fock.F:468-522 */
    {
        /* exchange pairs: 5 and 12 (IL|JK) first, 7 and 12 (IK|JL) */
        if (it == 5) {
            faar[ij] += r * daar[kl] * 4.0;
            faar[kl] += r * daar[ij] * 2.0;
        } else if (it == 7) {
            faar[kl] += r * daar[ij] * 4.0;
            faar[ij] += r * daar[kl] * 2.0;
        } else {
            faar[ij] += r * daar[kl] * 4.0;
            faar[kl] += r * daar[ij] * 4.0;
        }
        if (it == 5 || it == 12) {
            a = tri(i, l);
            b = tri(j, k);
            /* F(IL) from D(JK), then F(JK) from D(IL) */
            c1 = -r * daar[b], c2 = -r * daai[b], c3 = -r * dbar[b], c4 = -r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
            c1 = -r * daar[a], c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
            faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        }
        if (it == 7 || it == 12) {
            a = tri(i, k);
            b = tri(j, l);
            /* F(IK) from D(JL), then F(JL) from D(IK) */
            c1 = -r * daar[b], c2 = -r * daai[b], c3 = -r * dbar[b], c4 = -r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
            c1 = -r * daar[a], c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
            faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        }
        break;
    }
    case 8:  /* fock.F:282-316 */
    case 13: /* fock.F:530-584 */
    case 14: /* fock.F:593-647 */
    {
        if (it == 8) {
            faar[kl] += r * daar[ij] * 4.0;
            faar[ij] += r * daar[kl] * 2.0;
        } else {
            faar[ij] += r * daar[kl] * 4.0;
            faar[kl] += r * daar[ij] * 4.0;
        }
        if (it == 13 || it == 14) {
            a = tri(i, l);
            b = tri(k, j);
            /* F(IL) from D(KJ), then F(KJ) from D(IL) */
            c1 = -r * daar[b], c2 = r * daai[b], c3 = r * dbar[b], c4 = r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
            c1 = -r * daar[a], c2 = r * daai[a], c3 = r * dbar[a], c4 = r * dbai[a];
            faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        }
        a = tri(i, k);
        if (it == 13) {
            b = tri(j, l);
            /* F(IK) from D(JL), then F(JL) from D(IK) */
            c1 = -r * daar[b], c2 = -r * daai[b], c3 = -r * dbar[b], c4 = -r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
            c1 = -r * daar[a], c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
            faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        } else {
            b = tri(l, j);
            /* F(IK) from D(LJ), then F(LJ) from D(IK) */
            c1 = -r * daar[b], c2 = r * daai[b], c3 = r * dbar[b], c4 = r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
            c1 = -r * daar[a], c2 = r * daai[a], c3 = r * dbar[a], c4 = r * dbai[a];
            faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        }
        break;
    }
    case 9:  /* fock.F:324-364 */
    case 10: /* fock.F:372-412 */
    case 11: /* fock.F:420-460 */
    {
        const double s = it == 9 ? -1.0 : 1.0;  /* sign of the imaginary Coulomb-pair terms */
        c1 = r * daar[kl] * 3.0, c2 = s * r * daai[kl], c3 = s * r * dbar[kl], c4 = s * r * dbai[kl];
        faar[ij] += c1, faai[ij] += c2, fbar[ij] += c3, fbai[ij] += c4;
        c1 = r * daar[ij] * 3.0, c2 = s * r * daai[ij], c3 = s * r * dbar[ij], c4 = s * r * dbai[ij];
        faar[kl] += c1, faai[kl] += c2, fbar[kl] += c3, fbai[kl] += c4;
        if (it == 9) {
            a = tri(i, l);
            b = tri(j, k);
            /* F(IL) from D(JK) (FCABR, FCABI), F(JK) from D(IL), real part only */
            c1 = -r * daar[b], c2 = r * daai[b], c3 = -r * dbar[b], c4 = r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] -= c4;
            faar[b] += -r * daar[a] * 2.0;
        } else if (it == 10) {
            a = tri(i, k);
            b = tri(j, l);
            /* F(IK) from D(JL), real part only, then F(JL) from D(IK) */
            faar[a] += -r * daar[b] * 2.0;
            c1 = -r * daar[a], c2 = -r * daai[a], c3 = -r * dbar[a], c4 = r * dbai[a];
            faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] -= c4;
        } else {
            a = tri(i, k);
            b = tri(j, l);
            /* F(IK) from D(JL), then F(JL) from D(IK), real part only */
            c1 = -r * daar[b], c2 = -r * daai[b], c3 = -r * dbar[b], c4 = r * dbai[b];
            faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] -= c4;
            faar[b] += -r * daar[a] * 2.0;
        }
        break;
    }
    default:
        break;
    }
}

/* The skeleton Fock sets of MFDFOCK over records 0..nrec-1 (file class
 * rec_file, type rec_it, rec_nt integrals in order): records of files above
 * mfil (and the Gaunt file 4) are not read.  dens and fock hold nmat sets of
 * four arrays of nsc(nsc+1)/2 elements; fock is overwritten.  Returns 0, or
 * 1 for a label outside 1..nsc (fock then holds the records before it). */
int orc_fock_skeleton(long nrec, const int* rec_file, const int* rec_it, const long* rec_nt,
                      const double* rint, const int* label2, const int* label1, int mfil, int nsc,
                      int nmat, const double* dens, double* fock) {
    const long n = (long)nsc * (nsc + 1) / 2;
    for (long x = 0; x < 4L * n * nmat; ++x) fock[x] = 0.0;
    long off = 0;
    for (int file = 1; file <= mfil && file <= 3; ++file) {
        off = 0;
        for (long r = 0; r < nrec; ++r) {
            const long nt = rec_nt[r];
            if (rec_file[r] == file) {
                for (long t = 0; t < nt; ++t) {
                    const unsigned u2 = (unsigned)label2[off + t], u1 = (unsigned)label1[off + t];
                    const long i = u2 >> 16, j = u2 & 0xFFFF, k = u1 >> 16, l = u1 & 0xFFFF;
                    if (i < 1 || i > nsc || j < 1 || j > nsc || k < 1 || k > nsc || l < 1 || l > nsc)
                        return 1;
                    for (int s = 0; s < nmat; ++s)
                        fock_one(rec_it[r], i, j, k, l, rint[off + t], dens + 4 * n * s, fock + 4 * n * s, n);
                }
            }
            off += nt;
        }
    }
    return 0;
}

/* One Gaunt integral of type it (GAUNT, source/tmoone/gaunt.F): returns 1
 * for a type GAUNT rejects (gaunt.F:25-28, Q2JOB class 6). */
static int gaunt_one(int it, long i, long j, long k, long l, double r, const double* d, double* f,
                     long n) {
    const double *daar = d, *dbar = d + n, *daai = d + 2 * n, *dbai = d + 3 * n;
    double *faar = f, *fbar = f + n, *faai = f + 2 * n, *fbai = f + 3 * n;
    long a, b, c, e;
    double c1, c2, c3, c4;
    switch (it) {
    case 2: /* gaunt.F:41-76, I = K > J = L */
        a = tri(i, j), b = tri(i, k), c = tri(j, l);
        c1 = -r * daar[a] * 3.0, c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
        faar[a] -= c1, faai[a] -= c2, fbar[a] -= c3, fbai[a] -= c4;
        c1 = -r * daar[b] * 3.0, c2 = r * daai[b], c3 = r * dbar[b], c4 = r * dbai[b];
        faar[c] -= c1, faai[c] -= c2, fbar[c] -= c3, fbai[c] -= c4;
        c1 = -r * daar[c] * 3.0, c2 = r * daai[c], c3 = r * dbar[c], c4 = r * dbai[c];
        faar[b] -= c1, faai[b] -= c2, fbar[b] -= c3, fbai[b] -= c4;
        return 0;
    case 10: /* gaunt.F:84-124, I = K > J > L */
    case 11: /* gaunt.F:132-172, I > K > J = L */
        a = tri(k, l), b = tri(i, j), c = tri(i, k), e = tri(j, l);
        c1 = -r * daar[a] * 3.0, c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
        faar[b] -= c1, faai[b] -= c2, fbar[b] -= c3, fbai[b] -= c4;
        c1 = -r * daar[b] * 3.0, c2 = -r * daai[b], c3 = -r * dbar[b], c4 = -r * dbai[b];
        faar[a] -= c1, faai[a] -= c2, fbar[a] -= c3, fbai[a] -= c4;
        if (it == 10) {
            faar[c] -= -r * daar[e] * 6.0;
            /* FCABR, FCABI: FBAR -= FCABR, FBAI += FCABI */
            c1 = -r * daar[c] * 3.0, c2 = r * daai[c], c3 = -r * dbar[c], c4 = r * dbai[c];
            faar[e] -= c1, faai[e] -= c2, fbar[e] -= c3, fbai[e] += c4;
        } else {
            c1 = -r * daar[e] * 3.0, c2 = r * daai[e], c3 = r * dbar[e], c4 = -r * dbai[e];
            faar[c] -= c1, faai[c] -= c2, fbar[c] -= c3, fbai[c] += c4;
            faar[e] -= -r * daar[c] * 6.0;
        }
        return 0;
    case 13: /* gaunt.F:180-228, I > K > J > L */
        a = tri(i, l), b = tri(k, j), c = tri(i, k), e = tri(j, l);
        c1 = -r * daar[b] * 3.0, c2 = -r * daai[b], c3 = -r * dbar[b], c4 = -r * dbai[b];
        faar[a] -= c1, faai[a] -= c2, fbar[a] -= c3, fbai[a] -= c4;
        c1 = -r * daar[a] * 3.0, c2 = -r * daai[a], c3 = -r * dbar[a], c4 = -r * dbai[a];
        faar[b] -= c1, faai[b] -= c2, fbar[b] -= c3, fbai[b] -= c4;
        c1 = -r * daar[e] * 3.0, c2 = r * daai[e], c3 = r * dbar[e], c4 = r * dbai[e];
        faar[c] -= c1, faai[c] -= c2, fbar[c] -= c3, fbai[c] -= c4;
        c1 = -r * daar[c] * 3.0, c2 = r * daai[c], c3 = r * dbar[c], c4 = r * dbai[c];
        faar[e] -= c1, faai[e] -= c2, fbar[e] -= c3, fbai[e] -= c4;
        return 0;
    case 14: /* gaunt.F:236-284, I > K > L > J */
        a = tri(i, l), b = tri(k, j), c = tri(i, k), e = tri(l, j);
        c1 = r * daar[b] * 3.0, c2 = r * daai[b], c3 = r * dbar[b], c4 = r * dbai[b];
        faar[a] += c1, faai[a] += c2, fbar[a] += c3, fbai[a] += c4;
        c1 = r * daar[a] * 3.0, c2 = r * daai[a], c3 = r * dbar[a], c4 = r * dbai[a];
        faar[b] += c1, faai[b] += c2, fbar[b] += c3, fbai[b] += c4;
        c1 = -r * daar[e] * 3.0, c2 = -r * daai[e], c3 = -r * dbar[e], c4 = -r * dbai[e];
        faar[c] -= c1, faai[c] -= c2, fbar[c] -= c3, fbai[c] -= c4;
        c1 = r * daar[c] * 3.0, c2 = r * daai[c], c3 = r * dbar[c], c4 = r * dbai[c];
        faar[e] += c1, faai[e] += c2, fbar[e] += c3, fbai[e] += c4;
        return 0;
    default:
        return 1;
    }
}

/* MFDBREIT (source/tmoone/mfdbreit.F:50-138): the Gaunt contributions of the
 * file-4 records (SRTBREI/SRTBREL) added to the Fock sets, which are zeroed
 * first unless accumulate (BREIT, after MFDFOCK; with ONLYBRT MFDBREIT clears
 * them itself, mfdbreit.F:50-65).  Returns 0, 1 for a label outside 1..nsc, 2 for a type
 * GAUNT rejects. */
int orc_fock_gaunt(long nrec, const int* rec_file, const int* rec_it, const long* rec_nt,
                   const double* rint, const int* label2, const int* label1, int nsc, int nmat,
                   int accumulate, const double* dens, double* fock) {
    const long n = (long)nsc * (nsc + 1) / 2;
    if (!accumulate)
        for (long x = 0; x < 4L * n * nmat; ++x) fock[x] = 0.0;
    long off = 0;
    for (long r = 0; r < nrec; ++r) {
        const long nt = rec_nt[r];
        if (rec_file[r] == 4) {
            for (long t = 0; t < nt; ++t) {
                const unsigned u2 = (unsigned)label2[off + t], u1 = (unsigned)label1[off + t];
                const long i = u2 >> 16, j = u2 & 0xFFFF, k = u1 >> 16, l = u1 & 0xFFFF;
                if (i < 1 || i > nsc || j < 1 || j > nsc || k < 1 || k > nsc || l < 1 || l > nsc)
                    return 1;
                for (int s = 0; s < nmat; ++s)
                    if (gaunt_one(rec_it[r], i, j, k, l, rint[off + t], dens + 4 * n * s, fock + 4 * n * s, n))
                        return 2;
            }
        }
        off += nt;
    }
    return 0;
}
