// rt_internal.h -- internal structures of the GB300 rotran library.
//
// Data layout in device memory (planar complex: plane 0 = re, 1 = im):
//
//   AO order      AO functions are renumbered block-major ("sorted order"):
//                 blocks = component (L, S) x irrep (1 or 4), each block in
//                 increasing reference index.  The L functions occupy sorted
//                 positions [0, nL) and the S functions [nL, n).
//   pair order    the pq blocks rotran transforms (LL pairs, and SS pairs
//                 when S functions exist; makind.F:70-90) grouped by
//                 (class, pair irrep), inside a group in increasing
//                 p(p-1)/2+q.  P = number of pairs.
//   buckets       the integral records sorted by pq bucket (value + (r,s)),
//                 one entry per (pq, rs) direction of every stored integral
//   A1            (stage A, per pair chunk) the GEMM1 operand G_pq(r,s),
//                 r in an AO block, s in its partner block (both r<->s
//                 orders: the full symmetric matrix of pair pq), expanded
//                 from the buckets: [r][pq][s] FP64, or BF16 digit slices
//   HA            (stage A, per pair chunk) [plane][r][b][pq]: sum_s G_pq(r,s) QA(s,b)
//   RI            (stage A) [plane][a][b][pq]: sum_r conj(QA(r,a)) HA(r,b)
//   Hp            [plane][ij][pq]: (pq| I J) = RI(I,J) + s_IJ RI(Jbar,Ibar)
//                 for the K(K+1) Kramers-unique spinor pairs (the "sort /
//                 transpose" between the two halves)
//   M3            (stage B, per ij chunk, per component block)
//                 [p][ij][plane][q]: Hp expanded to the symmetric n_c x n_c matrix
//   RK            [plane][p][ij][k]: sum_q M_ij(p,q) QA(q,k)
//   RLR           [plane][l][ij][k]: sum_p conj(QA(p,l)) RK(p,k)
//   RL(K,L) = RLR(K,L) + s_KL RLR(Lbar,Kbar) gives the complete integrals
//   (I J | K L) from which the MDCINT records are selected.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/rotran_gb300.h"
#include "rt_kernels.h"

namespace rt {

#define RT_CUDA(call)                                                                   \
    do {                                                                                \
        cudaError_t e__ = (call);                                                       \
        if (e__ != cudaSuccess) throw rt::Error(RT_ERR_PROGRAM, std::string("CUDA: ") + \
                                                cudaGetErrorString(e__) + " at " #call); \
    } while (0)

struct Error {
    int code;
    std::string msg;
    Error(int c, std::string m) : code(c), msg(std::move(m)) {}
};

// message returned by rt_last_error(NULL) on the calling thread
void set_thread_error(const std::string& msg);

// A GEMM1 group: pairs of one pair-group against one r-block.
struct G1Group {
    int pg;          // pair group index
    int rblk;        // AO block of r
    int kblk;        // AO block of s (partner block)
    long long a_pp;  // offset of its operand in the expanded chunk buffer, per pair (elements)
    long long e_pp;  // offset of its row exponents, per pair
};

struct PairGroup {
    int cls;         // 0 = LL, 1 = SS, 2 = SL (Gaunt integrals)
    int gamma;       // pair irrep
    int start, size; // range in pair order
};

// One transform item of TRANS2's loop (trans2.F:73-74,230-238): barred spinor
// I of Kramers pair ikr, spinor J of pair jkr (barred: class 1; unbarred:
// classes 2, 3, 4), jkr <= ikr.
struct Item {
    int I, J;        // 0-based spinor indices
    int ikr, jkr;    // 1-based Kramers-pair indices
    int cls1;        // 1: J barred (class 1 record), 0: classes 2,3,4
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct Plan {
    int n = 0, nL = 0, nS = 0, m = 0, K = 0;
    int nblk = 0;
    std::vector<int> blk_start, blk_size, blk_comp, blk_irr;
    std::vector<int> ao_sorted;   // reference AO index (0-based) -> sorted position
    std::vector<int> ao_block;
    int P = 0;
    std::vector<PairGroup> pgroups;
    std::vector<int> pair_of_orig; // p(p-1)/2+q-1 -> pair order index or -1
    std::vector<int> pair_p, pair_q; // sorted AO positions of each pair (p >= q in reference order)
    std::vector<G1Group> g1;
    std::vector<std::vector<ExpandJob>> pg_jobs;   // expansion bands per pair group
    std::vector<long long> pg_a_pp;                // operand elements per pair (all groups)
    std::vector<long long> pg_e_pp;                // row exponents per pair
    int expand_kp_slices = -1;                     // slice count the jobs were laid out for
    // pq buckets are split by expansion job: bucket of (pair, job) =
    // pg_bbase[pg] + (pair - pg start) * pg_njobs[pg] + job
    std::vector<int> pg_njobs;
    std::vector<long long> pg_bbase;
    std::vector<int> jb_base, jb_band;             // [npg * nblk]: first job, band rows (-1: none)
    long long nbuckets = 0;
    std::vector<Item> items;      // K(K+1) items in TRANS2 order
    std::vector<int> cls1_rank;   // record position of each item within its class stream(s)
    int n_cls1 = 0, n_cls234 = 0;
    // expansion tables: per component block c (0 = L, 1 = S) the pair index
    // of (p, q) in component-local sorted positions, -1 if none
    // (Gaunt: row component c against the other component's columns)
    std::vector<int> pidx[2];
    int pidx_cols[2] = {0, 0};    // columns of pidx[c]: n_c (Coulomb) or n of the other component
    int ncomp[2] = {0, 0};
    int comp_off[2] = {0, 0};
};

struct Stage {
    int pair_chunk = 0;
    int item_chunk = 0;
};

// Host tables of the transform derived from the coefficients.
struct Work {
    std::vector<int4> items4;     // (I, J, Ibar, Jbar) per item
    std::vector<float> isign;     // sign(ITRMO(I) ITRMO(J))
    std::vector<double> pair_vmx; // VMX(p) VMX(q) per pair (trout.F:30)
    std::vector<EmitRec> recs;    // MDCINT records in item order
    std::vector<int> item_rec0;   // first record of each item
    long long cap[4] = {0, 0, 0, 0};   // element capacity per class
    long long nrec[4] = {0, 0, 0, 0};  // records per class
};

struct SplitState;  // rt_split.cu

// CUDA events around the GEMM kernel launches of one transform: their summed
// device time is the live duration of the dominant kernel class.
struct KTimer {
    cudaStream_t st = nullptr;
    std::vector<cudaEvent_t> ev;
    int used = 0;
    int launches = 0;
    double flops = 0.0;  // FLOPs the timed kernels executed
    double alg = 0.0;    // their algorithmic (one-product) FLOPs
    void reset(cudaStream_t s) { st = s; used = 0; launches = 0; flops = 0.0; alg = 0.0; }
    void begin() { mark(); }
    void end(double fl, double al) { mark(); ++launches; flops += fl; alg += al; }
    void mark() {
        if (used == (int)ev.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            ev.push_back(e);
        }
        cudaEventRecord(ev[used++], st);
    }
    double total_ms() const {
        double t = 0.0;
        for (int i = 0; i + 1 < used; i += 2) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, ev[i], ev[i + 1]) == cudaSuccess) t += ms;
        }
        return t;
    }
    ~KTimer() {
        for (auto e : ev) cudaEventDestroy(e);
    }
};

// Phase trace of a transform, on when RT_TRACE is set (and not "0") at
// rt_create: events on the context stream at each mark give the device time
// between marks, a steady clock the host time at which each mark was issued.
// Printed to stderr after the call, like rotran's per-step timing lines.
struct PhaseTrace {
    bool on = false;
    cudaStream_t st = nullptr;
    std::vector<cudaEvent_t> ev;
    std::vector<const char*> what;
    std::vector<double> host_ms;
    std::chrono::steady_clock::time_point t0;
    void reset(cudaStream_t s) {
        st = s;
        what.clear();
        host_ms.clear();
        t0 = std::chrono::steady_clock::now();
    }
    void mark(const char* w) {
        if (!on) return;
        const size_t i = what.size();
        if (i == ev.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return;
            ev.push_back(e);
        }
        cudaEventRecord(ev[i], st);
        what.push_back(w);
        host_ms.push_back(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
    void print(const char* title) const {
        if (!on || what.size() < 2) return;
        cudaEventSynchronize(ev[what.size() - 1]);
        std::fprintf(stderr, "rotran-gb300 %s trace: phase, device ms since the previous mark, host ms at the mark\n",
                     title);
        for (size_t i = 1; i < what.size(); ++i) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[i - 1], ev[i]);
            std::fprintf(stderr, "  %-34s %10.3f %10.3f\n", what[i], ms, host_ms[i]);
        }
    }
    ~PhaseTrace() {
        for (auto e : ev) cudaEventDestroy(e);
    }
};

}  // namespace rt

struct rt_ctx {
    rt_config cfg{};
    std::vector<int> ao_irrep;
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t cstream[4] = {};  // host <-> device copies in pieces
    cudaEvent_t ev[8] = {};
    bool have_coef = false;
    // set when an aborted GEMM could not confirm that its tensor-core work
    // and copies had finished: no further device work runs on the context
    bool unusable = false;
    // host copies of the tables
    std::vector<double> qa;   // n x m complex, column-major, interleaved
    std::vector<int> itrmo, kra, krb, ikrmo, imoras;  // in the internal spinor order
    std::vector<int> spin_user;  // internal spinor -> caller's spinor (0-based)
    rt::Plan plan;
    rt::Stage stage;
    rt::Work work;
    rt::SplitState* split = nullptr;
    rt::KTimer ktimer;
    rt::PhaseTrace trace;
    // records
    std::vector<int> rec_file, rec_it;
    std::vector<long long> rec_off, rec_nt;
    long long n_int = 0;     // integrals stored on device
    long long cap_int = 0;
    double* d_rint = nullptr;
    int* d_l2 = nullptr;
    int* d_l1 = nullptr;
    // the next record set queued by rt_queue_ao_records_bulk: host arrays
    // borrowed until the rt_transform that copies them returns
    struct RecordQueue {
        bool pending = false, issued = false;
        std::vector<int> file, it;
        std::vector<long long> nt;
        long long tot = 0;
        const double* rint = nullptr;
        const int* l2 = nullptr;
        const int* l1 = nullptr;
    } rq;
    cudaStream_t pstream[4] = {};  // the queued records' copies
    // staging for per-record calls
    std::vector<double> st_v;
    std::vector<int> st_l2, st_l1;
    double* h_pin_v = nullptr;
    int* h_pin_l2 = nullptr;
    int* h_pin_l1 = nullptr;
    size_t pin_cap = 0;
    // device arrays
    int* d_bcount = nullptr;      // bucket fill counters [P+1]
    long long* d_boff = nullptr;  // bucket offsets [P+1]
    double* d_bval = nullptr;     // bucket entries: value
    int* d_brs = nullptr;         // bucket entries: r<<16|s
    long long bucket_cap = 0;
    double* d_qap = nullptr;     // [s_sorted][plane*m + b]     (n x 2m)
    double* d_qah = nullptr;     // [(plane',a)][(plane,r)]     (2m x 2n)
    double* d_qar[2] = {nullptr, nullptr};  // per component: [(plane,q)][(plane',k)] (2nc x 2m)
    // Gaunt (Breit) transformation: the same operands built from QB (the
    // beta coefficients, QB(j) = -conj(QA(jbar)), QB(jbar) = conj(QA(j)))
    double* d_qbh = nullptr;     // like d_qah
    double* d_qbhS = nullptr;    // like d_qah with the large-component columns zero
    double* d_qbr[2] = {nullptr, nullptr};  // like d_qar
    // second bucket level: (pq, expansion job) buckets
    long long* d_jstart = nullptr;
    int* d_jcount = nullptr;
    double* d_jval = nullptr;
    int* d_jrs = nullptr;
    long long bucket_n = 0;  // (pq, job) buckets allocated
    double* d_ha = nullptr;
    size_t ha_len = 0;  // doubles in d_ha
    double* d_ri = nullptr;
    double* d_hp = nullptr;
    double* d_rl_all = nullptr;  // Gaunt: RL of every item, [item][K][L] (re, im)
    double* d_m3 = nullptr;
    double* d_rk = nullptr;
    double* d_rlr = nullptr;
    double* d_vmx = nullptr;
    int* d_tab = nullptr;        // device copies of small index tables
    size_t tab_bytes = 0;
    int* d_items = nullptr;
    // output
    int* d_cnt = nullptr;        // per record (chunk) counts
    int* d_pad_idx = nullptr;
    double* d_pad_val = nullptr;
    int* d_hdr[4] = {};
    int* d_oidx[4] = {};
    double* d_oval[4] = {};
    long long out_nrec[4] = {}, out_nz[4] = {}, out_cap[4] = {};
    // caller's host buffers the next transform streams each class into
    // (rt_set_result_host): elements copied as their item chunk completes
    // the Fock builds' work lists (records in chunks; [0] files 1..MFIL for
    // rt_fock_skeleton, [1] file 4 for rt_fock_gaunt), kept while the
    // records are unchanged (fock_gen == gen)
    void* d_fock_chunks[2] = {nullptr, nullptr};
    long long n_fock_chunks[2] = {0, 0};
    unsigned long long fock_gen[2] = {~0ull, ~0ull};
    bool host_on = false;
    bool host_defer = false;     // rt_transform returns before its last copies land
    bool host_inflight = false;  // copies of the last transform still on cstream[0]
    int* host_idx[4] = {};
    double* host_val[4] = {};
    long long host_cap[4] = {};
    unsigned long long* d_stat = nullptr;
    rt_stats stats{};
    size_t dev_bytes = 0, dev_peak = 0;
    std::vector<std::pair<void*, size_t>> allocs;
    // released per-call temporaries kept for the next call (still in allocs)
    std::vector<std::pair<void*, size_t>> pool;
    size_t pool_bytes = 0;
    bool transformed = false;
    unsigned long long gen = 0;  // input generation (coefficients, records)
};
