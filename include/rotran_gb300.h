/*
 * rotran_gb300.h -- C-ABI of the GB300 (sm_103a) implementation of MOLFDIR
 * rotran's Coulomb four-index transformation.
 *
 * The calls replace, inside a rotran driver, the sequence
 *   SR2INI / SORT1 / TRANS1 / SR2FLSH / TRANS2 / INITTWOE / PPSYM / EXITTWOE
 * of source/rotran/rotran.F:236-333.  The host keeps INIT, READIN, GETMOS
 * and COMSYM (rotran.F:42-45) and hands over the data those routines leave
 * in COMMON blocks: the spinor coefficients QA (/VECS/, vecs.inc:7), the
 * Kramers tables ITRMO/KRA/KRB/IKRMO (/REORD/, vecs.inc:11-12), the MDCINT
 * header orbital pairs, the /INPT/ sizes and the /TRES/ thresholds.
 *
 * Conventions
 *  - Every array is borrowed for the duration of the call only; the library
 *    copies what it needs.  A context owns its device memory and one CUDA
 *    stream and must not be shared between threads.
 *  - Complex numbers are two consecutive doubles (re, im), the memory layout
 *    of Fortran COMPLEX*16; matrices are column-major (Fortran order).
 *  - Spinor, AO and Kramers-pair indices are 1-based, as in the reference.
 *  - Every call returns an int status: 0 for success, otherwise the error
 *    class of Q2JOB (source/general/q2job.F:8-23) that the reference would
 *    have stopped with; rt_last_error() gives the message.  Nothing aborts
 *    inside the library and no call falls back to a CPU path: without a
 *    usable sm_103a device, rt_create fails with RT_ERR_PROGRAM.
 */
#ifndef ROTRAN_GB300_H
#define ROTRAN_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes = Q2JOB classes (q2job.F:8-23) */
#define RT_OK 0
#define RT_ERR_EOF 1      /* missing or truncated input data */
#define RT_ERR_USER 2     /* inconsistent input */
#define RT_ERR_DIM 3      /* a size exceeds what the library supports */
#define RT_ERR_INTERNAL 4 /* internal dimension error */
#define RT_ERR_MISMATCH 5 /* non-matching parameters between calls */
#define RT_ERR_PROGRAM 6  /* any other failure (CUDA error, Kramers check) */

#define RT_PREC_FP64 0       /* plain FP64 arithmetic on the CUDA cores */
#define RT_PREC_SPLIT_BF16 1 /* BF16 slices on the tensor cores, FP64 recombination */

typedef struct rt_ctx rt_ctx;

/* Sizes and options: /INPT/ (inpt.inc:1-8), /TRES/ (thres.inc:1-2). */
typedef struct rt_config {
    int nsc;          /* NSC: scalar AO functions transformed */
    int nsc1;         /* NSC1: large-component functions, 1..NSC1; S = NSC1+1..NSC */
    int nsp;          /* NSP: active spinors */
    int nkr;          /* NKR: Kramers pairs, NSP = 2*NKR */
    int mfil;         /* MFIL: SRT files read (1 LL, 2 +SS|LL, 3 +SS|SS), readin.F:83-84 */
    int breit;        /* BREIT (readin.F:17, default .FALSE. at readin.F:80): 0 Coulomb; 1 Gaunt, file 4 (SL|SL)
                         only, result stream MDBINT (rt_transform only; needs
                         0 < NSC1 < NSC; batches and rt_adjoint refuse it) */
    double thrgen;    /* THRGEN (readin.F:93) */
    double throut;    /* THROUT (readin.F:94): |x| > THROUT is written to MDCINT */
    int precision;    /* RT_PREC_FP64 or RT_PREC_SPLIT_BF16 */
    int slices;       /* split path: BF16 slices per operand, 2..6 (0: default 5) */
    int n_irrep;      /* 1, or 4: AO functions carry the labels in ao_irrep and
                         (pq|rs) vanishes unless irr(p)^irr(q) == irr(r)^irr(s) */
    const int* ao_irrep; /* NSC labels 0..n_irrep-1 (NULL when n_irrep == 1) */
    long long mem_budget; /* device bytes the context may use (0: 85% of the free
                             memory plus the work arena the context already holds) */
    int half_buckets; /* 1: bucket every integral under its LABEL1 pair only, as
                         rotran's SORT1 does (sort1.F:78-142), so the half-
                         transformed values, THRGEN's screen and NHALFT are
                         rotran's, and assemble each record from the two halves
                         as OUTPP1/OUTPP2/PPSYM do, THROUT on each half; holds
                         NKR(NKR+1)*NSP^2*16 more bytes (every item's result).
                         Always on for BREIT.  0 (default): each integral
                         under both of its pairs, complete sums, no extra
                         memory; equal to rotran's output at THRGEN <= 1e-16 */
} rt_config;

typedef struct rt_stats {
    long long nhalft;       /* half-transformed values kept by the THRGEN screen */
    long long nfinal[4];    /* MDCINT elements per class (NFINAL1..4, rotran.F:345) */
    long long nrec[4];      /* MDCINT records per class */
    double ms_upload, ms_scatter, ms_first, ms_second, ms_output, ms_total;
    double flops_algorithmic; /* algorithmic FLOPs of the transform (dense-block count) */
    long long device_bytes;   /* peak device memory held by the context */
    int gpu_launches;         /* kernels launched by the last rt_transform */
    int gemm_launches;        /* of which GEMM (half-transformation) kernels */
    double ms_gemm;           /* summed device time of the GEMM kernels */
    double flops_gemm_executed; /* FLOPs the GEMM kernels executed (slice products included) */
    double flops_gemm_algorithmic; /* the same GEMMs counted once (2 M N K each) */
} rt_stats;

/* Sizes of a transformation, computed on the host without a device: the
 * pq blocks transformed (makind.F:58-112), device bytes of the main arrays,
 * MDCINT records and an upper bound of their elements per class. */
typedef struct rt_plan_info {
    long long npairs;          /* pq blocks transformed */
    long long nitems;          /* Kramers-unique spinor pairs, NKR*(NKR+1) */
    long long expand_bytes_per_pair; /* FP64 G_pq(r,s) operand of one pq block */
    long long hp_bytes;        /* half-transformed integrals */
    long long nrec[4];         /* MDCINT records per class */
    long long elem_cap[4];     /* upper bound of MDCINT elements per class */
    double flops_algorithmic;  /* algorithmic FLOPs (dense-block count) */
} rt_plan_info;

int rt_plan(const rt_config* cfg, rt_plan_info* out);

/* Create a context on the current CUDA device (replaces the work-array set-up
 * of rotran.F:74-231).  Fails with RT_ERR_PROGRAM if no sm_103a device. */
int rt_create(rt_ctx** out, const rt_config* cfg);

/* Spinor coefficients and Kramers tables (GETMOS, getmos.F:3-242;
 * KRAMERS, kramers.F:3-165).  qa: QA(ld_qa, NSP) COMPLEX*16, rows 1..NSC
 * used; itrmo/ikrmo: NSP entries; kra/krb: NKR spinor indices of the
 * unbarred/barred member of each pair; imoras_pairs: 2*NKR orbital numbers
 * written to the MDCINT header (inittwoe.F:21-23). */
int rt_set_coefficients(rt_ctx* ctx, const double* qa, int ld_qa, const int* itrmo,
                        const int* kra, const int* krb, const int* ikrmo,
                        const int* imoras_pairs);

/* One SRTTW/SRTLB record pair as GETTW reads it (gettw.F:15-29): nt unscaled
 * integrals of type itype from file file_class (1 = SRTTWLL, 2 = SRTTWSL
 * (SS|LL), 3 = SRTTWSS); label2 = I<<16|K of the first pair, label1 =
 * L<<16|N of the second (the pq bucket of sort1.F:124-142).  Records of
 * files above MFIL are accepted and ignored, as SORT1 does not read them. */
int rt_add_ao_records(rt_ctx* ctx, int file_class, int nt, int itype, const double* rint,
                      const int* label2, const int* label1);

/* Many records at once: nrec records, record r holds nt[r] integrals of
 * type itype[r] from file file_class[r]; rint/label2/label1 are the records
 * concatenated and may be host or device memory of the current device. */
int rt_add_ao_records_bulk(rt_ctx* ctx, long long nrec, const int* file_class, const long long* nt,
                           const int* itype, const double* rint, const int* label2,
                           const int* label1);

/* Read SRTTWLL/SRTLBLL, SRTTWSL/SRTLBSL, SRTTWSS/SRTLBSS (gfortran
 * sequential unformatted, 4-byte markers) from directory dir, files
 * 1..MFIL, as SORT1 does (sort1.F:60-147). */
int rt_read_srt_files(rt_ctx* ctx, const char* dir);

/* Read the MPI version's pq-sorted integral files of ranks 0..nranks-1
 * from directory dir (replaces GETPQ's input, getpq.F:57-125, and its set-up
 * in rotran.par.F:430-506): SRTPQLN[.r], one sequential record LRECCO,
 * IRECL, ILSTA, ILEND, ISSTA, ISEND; SRTPQIL[.r], LRECCO direct-access
 * records of IRECL bytes, each IPQL, NT, INXT, RBUF(NT) real*8,
 * LBUF(NT) I<<16|K (32-bit layout, mfdtwoe.par.F:344-352,919-926).  Rank
 * 0's files have no suffix.  Every record is read once: the INXT links must
 * chain each stream's records, newest first.  Records of an SL pq pair
 * (Breit) are skipped; each other entry is the integral (I K | pq) of type
 * INTTYP with the larger pair first (getpq.F:81-96), added as by
 * rt_add_ao_records (file class from the L/S types of the two pairs). */
int rt_read_srtpq_files(rt_ctx* ctx, const char* dir, int nranks);

/* No counterpart in the reference: the same parse without a context or a
 * device, for checks and tools.  nsc/nsc1 as in rt_config.  On return
 * *nrec = records (one per file class and type, at most 42) and *nint =
 * integrals; if *nint > cap, returns RT_ERR_DIM and copies nothing (call
 * with cap = 0 to size the arrays).  Otherwise fills file_class, itype, nt
 * (nrec entries) and rint, label2, label1 (nint entries).  Errors: message
 * in rt_last_error(NULL). */
int rt_srtpq_scan(const char* dir, int nranks, int nsc, int nsc1, long long cap, long long* nrec,
                  long long* nint, int* file_class, int* itype, long long* nt, double* rint,
                  int* label2, int* label1);

/* Drop all records added so far (a new integral set, same sizes). */
int rt_clear_ao_records(rt_ctx* ctx);

/* Queue the next record set (arguments as rt_add_ao_records_bulk) so that
 * its host->device copies overlap the next rt_transform: that call reads the
 * current records during its bucketing, then copies the queued ones into
 * the record arrays on streams of their own while its half-transformations
 * run, and returns with the queued set as the context's records (whatever
 * its outcome); its results are those of the records it started with.  The
 * arrays are borrowed until that rt_transform returns (pinned host memory
 * copies asynchronously).  Any other call that reads or changes the records
 * (rt_add_*, rt_clear_ao_records, rt_read_*, rt_adjoint, rt_fock_*,
 * rt_batch_create, a second rt_queue_ao_records_bulk) first makes the queued
 * set current synchronously; rt_batch_run refuses a context with a set
 * queued (RT_ERR_MISMATCH).  (No counterpart in the reference, which reads
 * its integral files once per run.) */
int rt_queue_ao_records_bulk(rt_ctx* ctx, long long nrec, const int* file_class, const long long* nt,
                             const int* itype, const double* rint, const int* label2, const int* label1);

/* Run the transformation: first half (TRANS1), sort/transpose, second half
 * (TRANS2) and particle-particle completion (PPSYM); the MDCINT records stay
 * in device memory until copied or written.  The previous result is
 * replaced: after a failed call there is none (rt_result_sizes,
 * rt_copy_result and rt_write_mdcint fail with RT_ERR_USER). */
int rt_transform(rt_ctx* ctx);

/* Adjoint of the transformation (no counterpart in the reference, which
 * has no derivatives).  With the integrals (ij|kl) of all NSP^4 spinor
 * quadruples defined from QA as rt_transform defines them, and
 *   E = sum_{ijkl} gamma(i,j,k,l) (ij|kl),
 * writes dedc(p,x) = dE/dRe QA(p,x) + i dE/dIm QA(p,x) (NSC x NSP COMPLEX*16,
 * column-major, leading dimension NSC) and *energy = E.  gamma is NSP^4
 * COMPLEX*16 in Fortran order, host or device memory; only its part
 * symmetric under pair exchange (ij)<->(kl) contributes.  The
 * half-transformed integrals are recomputed (without the THRGEN screen),
 * not taken from an earlier rt_transform.  Needs the context's records and
 * coefficients; runs in the context's precision (the split path puts the
 * density contraction on the tensor cores as well).  Device memory: the
 * density (16 NSP^4 bytes) plus the arrays of rt_transform. */
int rt_adjoint(rt_ctx* ctx, const double* gamma, double* dedc, double* energy);

/* tmoone's skeleton Fock matrices (MFDFOCK, source/tmoone/mfdfock.F:53-140,
 * with FOCK, source/tmoone/fock.F:1-656) from the context's integral
 * records of files 1..MFIL, on the GPU.  dens holds nmat (1: closed shell,
 * COMMON /DMT/; 2: closed then open shell, /DMT/ and /DOMT/) sets of four
 * lower-triangle arrays DAAR, DBAR, DAAI, DBAI of NSC(NSC+1)/2 elements each,
 * element (x,y), x >= y, at x(x-1)/2 + y - 1 (densfock.inc:4-5; the
 * reference's arrays are dimensioned N21 and use this leading part); fock
 * receives FAAR, FBAR, FAAI, FBAI (/FMT/, /FOMT/) in the same layout,
 * overwritten.  Host or device pointers.  The records are the ones rotran
 * transforms (rt_add_ao_records*, rt_read_srt_files; LABEL2 gives I, J and
 * LABEL1 K, L as in mfdfock.F:103-114); coefficients are not needed.  The
 * additions run in a different order than the reference's (FP64 atomics),
 * so the sums agree to rounding.  *ms_kernel (may be NULL) receives the
 * kernel's device milliseconds.  A label outside 1..NSC or a type outside
 * 1..14 fails with RT_ERR_USER. */
int rt_fock_skeleton(rt_ctx* ctx, int nmat, const double* dens, double* fock, double* ms_kernel);

/* tmoone's Gaunt contributions to the same Fock sets (MFDBREIT,
 * source/tmoone/mfdbreit.F:50-138, with GAUNT, source/tmoone/gaunt.F) from
 * the context's file-4 records (SRTBREI/SRTBREL, class 4 of
 * rt_add_ao_records*; rt_read_srt_files reads them for contexts created with
 * BREIT = 1).  Layouts as rt_fock_skeleton.  accumulate = 1 adds them to the
 * sets passed in fock (BREIT: after MFDFOCK, mfddriv.F:46); accumulate = 0
 * overwrites (ONLYBRT, mfddriv.F:42, where MFDBREIT clears the sets).  A
 * record type GAUNT does not accept (other than 2, 10, 11, 13, 14) fails
 * with RT_ERR_PROGRAM, as GAUNT's Q2JOB(6) does. */
int rt_fock_gaunt(rt_ctx* ctx, int nmat, const double* dens, double* fock, int accumulate,
                  double* ms_kernel);

/* Batched transforms (no counterpart in the reference, which runs one
 * transformation per process).  rt_batch_create plans every context as a
 * single chunk (all pair groups and Kramers items resident at once; fails
 * with RT_ERR_DIM when they do not all fit) and builds one grouped GEMM per
 * stage over all contexts.  rt_batch_run runs the transforms; its first call
 * times every grouped GEMM with 128- and 64-wide output tiles, keeps the
 * faster, and captures the whole sequence as a CUDA graph that later calls
 * replay.  With RT_TUNE_CACHE naming a file in the environment, the choices
 * are stored there under each stage's shape class (a flat JSON object), and
 * a batch whose stages are all in the file skips the timing runs
 * (ms_tune = 0).  The results are then read per context with rt_result_sizes /
 * rt_copy_result / rt_write_mdcint.  All contexts: same device, precision
 * RT_PREC_SPLIT_BF16, coefficients and records set before rt_batch_create
 * and left unchanged while the batch lives (RT_ERR_MISMATCH otherwise).
 * The batch keeps work arrays in its contexts: destroy it before any of
 * them. */
typedef struct rt_batch rt_batch;
typedef struct rt_batch_stats {
    int instances;
    int grouped_launches;  /* persistent grouped GEMM launches per run */
    int kernel_launches;   /* all kernels of one run */
    int graph_nodes;       /* nodes of the captured graph */
    int tile128, tile64;   /* grouped launches tuned to 128- / 64-wide tiles */
    double ms_last;        /* device time of the last run (graph launch) */
    double ms_tune;        /* device time of the two tuning runs (0: from the cache) */
    double flops_algorithmic;   /* summed algorithmic FLOPs of the transforms */
    double flops_gemm_executed; /* tensor FLOPs of the grouped GEMMs per run */
} rt_batch_stats;
int rt_batch_create(rt_batch** out, rt_ctx* const* ctxs, int count);
int rt_batch_run(rt_batch* b);
int rt_batch_get_stats(rt_batch* b, rt_batch_stats* out);
/* message of the last failed rt_batch_run (rt_batch_create: rt_last_error(NULL)) */
const char* rt_batch_last_error(rt_batch* b);
void rt_batch_destroy(rt_batch* b);

/* Sizes of the MDCINT record stream of the last transform (records without
 * header and terminator; nz = total elements). */
int rt_result_sizes(rt_ctx* ctx, long long* nrec, long long* nz);

/* Copy the record stream: hdr[3*nrec] = (IKR*IS, JKR*JS, NZ) in file order
 * (ppsym.F:89-91), idx[2*nz] = (INDK, INDL), val[2*nz] = (re, im). */
int rt_copy_result(rt_ctx* ctx, int* hdr, int* idx, double* val);

/* Stream the elements of the following rt_transform calls into caller-owned
 * host buffers, one per record class c = 0..3 (MDCINT classes 1..4):
 * idx[c] holds 2*cap[c] ints, val[c] 2*cap[c] doubles, in the order
 * rt_copy_result gives that class's elements.  Each item chunk's elements
 * are copied as soon as the chunk is done, overlapping the remaining work
 * (pinned buffers copy asynchronously); rt_transform returns with all of
 * them in place, and rt_copy_result(ctx, hdr, NULL, NULL) then gives the
 * headers.  A class with more elements than cap[c] fails the transform with
 * class 3.  NULL idx or val unregisters. */
int rt_set_result_host(rt_ctx* ctx, int* const* idx, double* const* val, const long long* cap);

/* With deferred = 1, rt_transform returns before the copies of its last
 * item chunk into the registered buffers have landed; they finish while the
 * caller (or the next rt_transform's first half, which never writes the
 * results) runs.  rt_result_host_wait waits for them; so do rt_copy_result,
 * rt_write_mdcint, rt_set_result_host, rt_set_result_host_deferred,
 * rt_adjoint, rt_batch_run and the next rt_transform before it writes
 * results again.  Default 0: rt_transform returns with every copy done. */
int rt_set_result_host_deferred(rt_ctx* ctx, int deferred);
int rt_result_host_wait(rt_ctx* ctx);

/* Write MDCINT (inittwoe.F:1-25, ppsym.F:89-91, exittwoe.F:1-10) as
 * a gfortran sequential unformatted file. */
int rt_write_mdcint(rt_ctx* ctx, const char* path, const char* datex10, const char* timex8);

int rt_get_stats(rt_ctx* ctx, rt_stats* out);
/* Message of the last failed call on ctx; with ctx == NULL, of the last
 * failed rt_create or rt_plan of the calling thread. */
const char* rt_last_error(rt_ctx* ctx);
void rt_destroy(rt_ctx* ctx);

/* C = A B (row-major FP64 host matrices, M x K times K x N) computed by the
 * split-precision engine of the transformation (BF16 digit slices on the
 * tensor cores, exact FP32 accumulation of the two leading slice products,
 * float-float recombination).  mode 0 slices both operands on the host;
 * mode 1 rounds A and B to float-float and slices them on the device, as
 * the intermediate quarter-transforms are; mode 2 slices FP64 rows of A on
 * the device, as the first quarter-transform does.  K <= 1024. */
int rt_split_dgemm(int M, int N, int K, const double* A, const double* B, double* C, int slices,
                   int mode);

/* No counterpart in the reference.  C = A B like rt_split_dgemm mode 2, on
 * DEVICE-resident row-major FP64 matrices (A M x K, B K x N, C M x N),
 * without allocating: all scratch (slices, scales, error flag, a
 * float-float copy of B) lives in one fixed 48 MiB device array per device,
 * so it suits callers that must not call cudaMalloc/cudaFree.  Needs
 *   256 + r(4M) + r(4N) + r(2 s M Kp) + r(2 s N Kp) + r(8 K N) <= 50331648
 * bytes, r() rounding up to 256 and Kp = K rounded up to 32 (M = N = K = 1024
 * fits at 6 slices); larger sizes and K > 1024 return RT_ERR_DIM with the
 * reason in rt_last_error(NULL).  `stream` is a cudaStream_t (NULL: the
 * legacy default stream); the call returns after the product is complete.
 * The first call on each device, with that device current, does a one-time
 * set-up (device address of the array, kernel attributes); make that first
 * call before any stream capture.  Every call shares the array and it keeps
 * the last call's contents: calls that overlap on the GPU (other host
 * threads, other streams) race and must be serialised by the caller. */
int rt_split_dgemm_noalloc(int M, int N, int K, const double* A, const double* B, double* C,
                           int slices, void* stream);

/* KRAMERS pairing check (kramers.F:26-131) on host data: finds the
 * time-reversal partner of every spinor (tolerance 1e-10), writes ITRMO and
 * the largest deviation; returns RT_ERR_PROGRAM, like the reference's
 * Q2JOB(6,...) stops, if a spinor has no partner or a partner needs a phase. */
int rt_kramers_check(int nsc, int nsp, const double* qa, const double* qb, int ld, int* itrmo,
                     double* difmax);

#ifdef __cplusplus
}
#endif
#endif
