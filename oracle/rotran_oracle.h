/* rotran_oracle.h -- interface of the CPU restatement of rotran's Coulomb
 * four-index transformation (test infrastructure; see rotran_oracle.c). */
#ifndef ROTRAN_ORACLE_H
#define ROTRAN_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int nsc;     /* NSC: scalar AO functions */
    int nsc1;    /* NSC1: large-component functions (1..nsc1) */
    int nsp;     /* NSP: active spinors */
    int nkr;     /* NKR: Kramers pairs, nsp == 2*nkr */
    int mfil;    /* number of SRT files read (1 LL, 2 +SS|LL, 3 +SS|SS) */
    int quater;  /* write class 4 (quaternionic group) */
    double thrgen, throut; /* &TRANTH thresholds */
    int nthreads;          /* OpenMP threads (0: runtime default) */
    long limit_pq;         /* >0: transform only the first limit_pq pq blocks */
    long limit_ij;         /* >0: only the first limit_ij TRANS2 pairs */
    const long* pq_select; /* optional list of pq blocks (p(p-1)/2+q) to transform */
    long n_pq_select;
    long fake_list_len;    /* >0 (timing samples): TRANS2 reads lists of this
                              length with synthetic values instead of TRANS1's */
    int breit;             /* 1: the Gaunt (Breit) transformation of the SL|SL
                              integrals of file 4 (SRTBREI) into MDBINT */
} orc_params;

typedef struct orc_result {
    long nrec;      /* MDCINT records, header and terminator excluded */
    int* hdr;       /* 3*nrec: IKR*IS, JKR*JS, NZ */
    long nz_total;
    int* idx;       /* 2*nz_total: INDK, INDL */
    double* val;    /* 2*nz_total: re, im */
    long nhalft;    /* half-transformed integrals kept (NHALFT) */
    long nskel;     /* transformed integrals written (NSKEL) */
    long nfinal[4]; /* final integrals per class (NFINAL1..4) */
    long npq_done, nij_done, nij_total;
    double t_first, t_second, t_pp; /* wall seconds of the three steps */
    int nijsiz, nc2;
} orc_result;

double orc_gettw_factor(int it);
int orc_inttyp(int imm, int jmm, int kmm, int lmm);
int orc_run(const orc_params* prm, const double* qa, const int* itrmo, const int* kra,
            const int* krb, const int* ikrmo, long nrec, const int* rec_file, const int* rec_it,
            const long* rec_nt, const double* rint, const int* label2, const int* label1,
            orc_result* out);
void orc_free(orc_result* r);

/* tmoone's skeleton Fock build (tmoone_fock_oracle.c) */
int orc_fock_skeleton(long nrec, const int* rec_file, const int* rec_it, const long* rec_nt,
                      const double* rint, const int* label2, const int* label1, int mfil, int nsc,
                      int nmat, const double* dens, double* fock);
int orc_fock_gaunt(long nrec, const int* rec_file, const int* rec_it, const long* rec_nt,
                   const double* rint, const int* label2, const int* label1, int nsc, int nmat,
                   int accumulate, const double* dens, double* fock);

#ifdef __cplusplus
}
#endif
#endif
