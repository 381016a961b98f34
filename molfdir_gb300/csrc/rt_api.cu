// rt_api.cu -- C-ABI entry points, planning and orchestration of the
// GB300 rotran transformation (replaces rotran.F:74-333).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "rt_internal.h"
#include "rt_kernels.h"
#include "rt_split.h"
#include "rt_access.h"

using namespace rt;

[[noreturn]] void rt::throw_dim(const char* what) { throw Error(RT_ERR_DIM, what); }

namespace {

template <class T>
T* dalloc(rt_ctx* c, size_t count) {
    if (count == 0) count = 1;
    void* p = nullptr;
    size_t bytes = count * sizeof(T);
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(RT_ERR_DIM, "device allocation of " + std::to_string(bytes) +
                                    " bytes failed (" + cudaGetErrorString(e) + ")");
    }
    c->allocs.push_back({p, bytes});
    c->dev_bytes += bytes;
    c->dev_peak = std::max(c->dev_peak, c->dev_bytes);
    return static_cast<T*>(p);
}

void dfree(rt_ctx* c, void* p) {
    if (!p) return;
    for (size_t i = 0; i < c->allocs.size(); ++i)
        if (c->allocs[i].first == p) {
            c->dev_bytes -= c->allocs[i].second;
            c->allocs.erase(c->allocs.begin() + i);
            break;
        }
    cudaFree(p);
}

// Per-call temporaries (tables, offsets, job lists: a few dozen small arrays
// per transform) come from a pool that keeps released blocks for the next
// call, so a repeated transform makes no cudaMalloc / cudaFree: cudaFree
// synchronises the device and a fresh cudaMalloc maps new pages.
constexpr size_t POOL_BLOCK_MAX = (size_t)16 << 20, POOL_TOTAL_MAX = (size_t)128 << 20;

void* tmp_alloc(rt_ctx* c, size_t bytes) {
    if (bytes == 0) bytes = 1;
    int best = -1;
    for (int i = 0; i < (int)c->pool.size(); ++i) {  // smallest block that fits, at most 2x
        const size_t b = c->pool[i].second;
        if (b >= bytes && b <= 2 * bytes + 4096 && (best < 0 || b < c->pool[best].second)) best = i;
    }
    if (best < 0) return dalloc<unsigned char>(c, bytes);
    void* p = c->pool[best].first;
    c->pool_bytes -= c->pool[best].second;
    c->pool.erase(c->pool.begin() + best);
    return p;
}

// Return temporaries; `settled` says no queued work still uses them.
void tmp_release(rt_ctx* c, const std::vector<void*>& tmp, bool settled) {
    for (void* p : tmp) {
        size_t bytes = 0;
        for (auto& a : c->allocs)
            if (a.first == p) bytes = a.second;
        if (!settled || bytes == 0 || bytes > POOL_BLOCK_MAX || c->pool_bytes + bytes > POOL_TOTAL_MAX) {
            dfree(c, p);
        } else {
            c->pool.push_back({p, bytes});
            c->pool_bytes += bytes;
        }
    }
}

template <class T>
void upload(rt_ctx* c, T*& dst, const std::vector<T>& v) {
    dfree(c, dst);
    dst = dalloc<T>(c, v.size());
    if (!v.empty())
        RT_CUDA(cudaMemcpyAsync(dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
}

void check_config(const rt_config* cfg) {
    if (!cfg) throw Error(RT_ERR_USER, "null configuration");
    if (cfg->nsc < 1 || cfg->nsc > 65535)
        throw Error(RT_ERR_DIM, "NSC must be in 1..65535 (16-bit integral labels)");
    if (cfg->nsc1 < 0 || cfg->nsc1 > cfg->nsc) throw Error(RT_ERR_USER, "NSC1 must be in 0..NSC");
    if (cfg->nkr < 1 || cfg->nsp != 2 * cfg->nkr)
        throw Error(RT_ERR_USER, "NSP must equal 2*NKR with NKR >= 1");
    if (cfg->nkr > cfg->nsc) throw Error(RT_ERR_USER, "more Kramers pairs than scalar functions");
    if (cfg->breit != 0 && cfg->breit != 1) throw Error(RT_ERR_USER, "BREIT must be 0 or 1");
    if (cfg->half_buckets != 0 && cfg->half_buckets != 1) throw Error(RT_ERR_USER, "half_buckets must be 0 or 1");
    if (cfg->breit) {
        // the Gaunt transformation (BREIT = .TRUE., MFIL = 0: rotran.F:48-57)
        // reads the SL|SL integrals of file 4; MFIL is not used
        if (cfg->nsc1 < 1 || cfg->nsc1 >= cfg->nsc)
            throw Error(RT_ERR_USER, "the Gaunt (Breit) transformation needs large and small component functions");
    } else {
        if (cfg->mfil < 1 || cfg->mfil > 3) throw Error(RT_ERR_USER, "MFIL must be 1, 2 or 3");
        if (cfg->mfil == 1 && cfg->nsc != cfg->nsc1)
            throw Error(RT_ERR_USER, "MFIL=1 transforms the large component only: NSC must equal NSC1");
    }
    if (cfg->precision != RT_PREC_FP64 && cfg->precision != RT_PREC_SPLIT_BF16)
        throw Error(RT_ERR_USER, "unknown precision");
    if (cfg->slices != 0 && (cfg->slices < 2 || cfg->slices > 6))
        throw Error(RT_ERR_USER, "slices must be 0 or 2..6");
    if (cfg->n_irrep != 1 && cfg->n_irrep != 4) throw Error(RT_ERR_USER, "n_irrep must be 1 or 4");
    // bucket entries pack (block, position) in 3 + 12 bits per index
    if (cfg->nsc1 > 4095 || cfg->nsc - cfg->nsc1 > 4095)
        throw Error(RT_ERR_DIM, "more than 4095 functions of one component");
    if (cfg->n_irrep == 4) {
        if (!cfg->ao_irrep) throw Error(RT_ERR_USER, "ao_irrep required when n_irrep == 4");
        for (int p = 0; p < cfg->nsc; ++p)
            if (cfg->ao_irrep[p] < 0 || cfg->ao_irrep[p] > 3)
                throw Error(RT_ERR_USER, "AO irrep labels must be 0..3");
    }
}

// AO blocks, pair groups and GEMM1 groups (the pq-block list of
// makind.F:58-112 and the block structure of the integral files).
void plan_ao(rt_ctx* c) {
    Plan& P = c->plan;
    const rt_config& cfg = c->cfg;
    P.n = cfg.nsc;
    P.nL = cfg.nsc1;
    P.nS = cfg.nsc - cfg.nsc1;
    P.m = cfg.nsp;
    P.K = cfg.nkr;
    const int nirr = cfg.n_irrep;
    auto irr = [&](int p) { return nirr == 1 ? 0 : c->ao_irrep[p]; };
    P.blk_start.clear(); P.blk_size.clear(); P.blk_comp.clear(); P.blk_irr.clear();
    P.ao_sorted.assign(P.n, -1);
    P.ao_block.assign(P.n, -1);
    std::vector<int> ao_pos(P.n, 0);
    int pos = 0;
    for (int comp = 0; comp < 2; ++comp) {
        int lo = comp == 0 ? 0 : P.nL, hi = comp == 0 ? P.nL : P.n;
        for (int g = 0; g < nirr; ++g) {
            int start = pos, cnt = 0;
            for (int p = lo; p < hi; ++p)
                if (irr(p) == g) {
                    P.ao_sorted[p] = pos++;
                    P.ao_block[p] = (int)P.blk_start.size();
                    ao_pos[p] = cnt++;
                }
            if (cnt == 0) continue;
            P.blk_start.push_back(start);
            P.blk_size.push_back(cnt);
            P.blk_comp.push_back(comp);
            P.blk_irr.push_back(g);
        }
    }
    P.nblk = (int)P.blk_start.size();
    P.ncomp[0] = P.nL;
    P.ncomp[1] = P.nS;
    P.comp_off[0] = 0;
    P.comp_off[1] = P.nL;
    // pairs: LL always, SS when S functions exist (MFIL >= 2 then)
    const long long ntri = (long long)P.n * (P.n + 1) / 2;
    P.pair_of_orig.assign(ntri, -1);
    struct PK { int cls, gamma; long long orig; int p, q; };
    std::vector<PK> pk;
    for (int p = 0; p < P.n; ++p)
        for (int q = 0; q <= p; ++q) {
            bool pl = p < P.nL, ql = q < P.nL;
            if (cfg.breit) {  // the SL blocks only (makind.F:91-95)
                if (pl == ql) continue;
                pk.push_back({2, irr(p) ^ irr(q), (long long)p * (p + 1) / 2 + q, p, q});
                continue;
            }
            if (pl != ql) continue;  // no SL blocks for Coulomb (makind.F:75)
            pk.push_back({pl ? 0 : 1, irr(p) ^ irr(q), (long long)p * (p + 1) / 2 + q, p, q});
        }
    std::stable_sort(pk.begin(), pk.end(), [](const PK& a, const PK& b) {
        if (a.cls != b.cls) return a.cls < b.cls;
        if (a.gamma != b.gamma) return a.gamma < b.gamma;
        return a.orig < b.orig;
    });
    P.P = (int)pk.size();
    P.pair_p.resize(P.P);
    P.pair_q.resize(P.P);
    P.pgroups.clear();
    for (int i = 0; i < P.P; ++i) {
        P.pair_of_orig[pk[i].orig] = i;
        P.pair_p[i] = pk[i].p;
        P.pair_q[i] = pk[i].q;
        if (P.pgroups.empty() || P.pgroups.back().cls != pk[i].cls || P.pgroups.back().gamma != pk[i].gamma)
            P.pgroups.push_back({pk[i].cls, pk[i].gamma, i, 0});
        P.pgroups.back().size++;
    }
    // GEMM1 groups: which r blocks meet each pair group, and their partner block
    P.g1.clear();
    long long base = 0;
    for (int g = 0; g < (int)P.pgroups.size(); ++g) {
        const PairGroup& pg = P.pgroups[g];
        for (int rb = 0; rb < P.nblk; ++rb) {
            int comp = P.blk_comp[rb];
            bool present;
            if (pg.cls == 2) present = true;                          // (SL|SL): r in L or S
            else if (pg.cls == 0) present = comp == 0 || cfg.mfil >= 2;   // (LL|LL), (LL|SS)
            else present = comp == 0 ? cfg.mfil >= 2 : cfg.mfil >= 3; // (SS|LL), (SS|SS)
            if (!present) continue;
            // partner block of s: the same component (Coulomb) or the other
            // one (Gaunt: G_pq(r,s) couples an L and an S function)
            const int kcomp = pg.cls == 2 ? 1 - comp : comp;
            int kb = -1;
            for (int b = 0; b < P.nblk; ++b)
                if (P.blk_comp[b] == kcomp && P.blk_irr[b] == (P.blk_irr[rb] ^ pg.gamma)) kb = b;
            if (kb < 0) continue;
            P.g1.push_back({g, rb, kb, 0, 0});
        }
    }
    (void)base;
    // expansion tables per row component: columns of the same component
    // (Coulomb) or of the other one (Gaunt)
    for (int comp = 0; comp < 2; ++comp) {
        const int oc = cfg.breit ? 1 - comp : comp;
        int nc = P.ncomp[comp], off = P.comp_off[comp];
        int ncol = P.ncomp[oc], coff = P.comp_off[oc];
        P.pidx_cols[comp] = ncol;
        P.pidx[comp].assign((size_t)nc * ncol, -1);
        // sorted position -> reference index
        std::vector<int> ref_of(P.n);
        for (int p = 0; p < P.n; ++p) ref_of[P.ao_sorted[p]] = p;
        for (int a = 0; a < nc; ++a)
            for (int b = 0; b < ncol; ++b) {
                int p = ref_of[off + a], q = ref_of[coff + b];
                int hi = std::max(p, q), lo = std::min(p, q);
                P.pidx[comp][(size_t)a * ncol + b] = P.pair_of_orig[(long long)hi * (hi + 1) / 2 + lo];
            }
    }
    (void)ao_pos;
}

// Expansion bands of every pair group and the per-pair layout of the GEMM1
// operand buffer (FP64 rows, or BF16 slices when nslices > 0).
void plan_expand(rt_ctx* c, int nslices) {
    Plan& P = c->plan;
    if (P.expand_kp_slices == nslices) return;
    const int npg = (int)P.pgroups.size();
    P.pg_jobs.assign(npg, {});
    P.pg_a_pp.assign(npg, 0);
    P.pg_e_pp.assign(npg, 0);
    P.jb_base.assign((size_t)npg * P.nblk, -1);
    P.jb_band.assign((size_t)npg * P.nblk, 1);
    for (auto& gg : P.g1) {
        const int nr = P.blk_size[gg.rblk], nk = P.blk_size[gg.kblk];
        const int kp = (nk + 31) / 32 * 32;
        gg.a_pp = P.pg_a_pp[gg.pg];
        gg.e_pp = P.pg_e_pp[gg.pg];
        // bands of at most 48 KB of FP64 G_pq(r,s): several CTAs per SM
        const int band = std::max(1, std::min(nr, (int)(49152 / (8 * nk))));
        P.jb_base[(size_t)gg.pg * P.nblk + gg.rblk] = (int)P.pg_jobs[gg.pg].size();
        P.jb_band[(size_t)gg.pg * P.nblk + gg.rblk] = band;
        for (int r0 = 0; r0 < nr; r0 += band) {
            ExpandJob j;
            j.rblk = gg.rblk;
            j.r_lo = r0;
            j.r_hi = std::min(nr, r0 + band);
            j.nr = nr;
            j.nk = nk;
            j.kp = kp;
            j.out_pp = gg.a_pp;
            j.exp_pp = gg.e_pp;
            P.pg_jobs[gg.pg].push_back(j);
        }
        P.pg_a_pp[gg.pg] += nslices ? (long long)nslices * nr * kp : (long long)nr * nk;
        P.pg_e_pp[gg.pg] += nr;
    }
    P.pg_njobs.assign(npg, 0);
    P.pg_bbase.assign(npg, 0);
    long long nb = 0;
    for (int g = 0; g < npg; ++g) {
        P.pg_njobs[g] = (int)P.pg_jobs[g].size();
        P.pg_bbase[g] = nb;
        nb += (long long)P.pgroups[g].size * P.pg_njobs[g];
    }
    if (nb >= (1LL << 31)) throw Error(RT_ERR_DIM, "more than 2^31 expansion buckets");
    for (int g = 0; g < npg; ++g)
        if (P.pg_njobs[g] > 1024) throw Error(RT_ERR_DIM, "more than 1024 expansion bands per pair");
    P.nbuckets = nb;
    P.expand_kp_slices = nslices;
}

// Size of the canonical element set of a record (see in_set in rt_kernels.cu).
long long set_size(int cls, int i, int j, int K, bool all) {
    if (all || cls == 3) return (long long)K * K;
    long long rank = (long long)i * (i - 1) / 2 + j;
    if (cls == 0) return i == j ? (long long)i * (i + 1) / 2 : 2 * rank - (i - 1);
    return rank;
}

struct DeviceTabs {
    unsigned char* pq_read;
    int *pair_of_orig, *pair_group, *pg_start, *pg_size, *ao_block, *ao_pos, *blk_size, *g1_of,
        *g1_kblk, *jb_base, *jb_band, *pg_njobs;
    long long* pg_bbase;
};

}  // namespace

// ---------------------------------------------------------------------------
// plan + tables that depend on the coefficients
// ---------------------------------------------------------------------------
static Work& W(rt_ctx* c) { return c->work; }

// ---------------------------------------------------------------------------
// device state
// ---------------------------------------------------------------------------
static void build_coef_device(rt_ctx* c) {
    Plan& P = c->plan;
    const int n = P.n, m = P.m;
    // QA in sorted AO order, planar
    std::vector<double> qr((size_t)n * m), qi((size_t)n * m);  // [sorted p][i]
    for (int p = 0; p < n; ++p)
        for (int i = 0; i < m; ++i) {
            qr[(size_t)P.ao_sorted[p] * m + i] = c->qa[2 * ((size_t)p + (size_t)i * n)];
            qi[(size_t)P.ao_sorted[p] * m + i] = c->qa[2 * ((size_t)p + (size_t)i * n) + 1];
        }
    // GEMM1 B: [s][plane*m + b]
    std::vector<double> qap((size_t)n * 2 * m);
    for (int s = 0; s < n; ++s)
        for (int b = 0; b < m; ++b) {
            qap[(size_t)s * 2 * m + b] = qr[(size_t)s * m + b];
            qap[(size_t)s * 2 * m + m + b] = qi[(size_t)s * m + b];
        }
    // GEMM2/4 A: [(plane',a)][(plane,r)] = [[QAr^T, QAi^T], [-QAi^T, QAr^T]]
    std::vector<double> qah((size_t)2 * m * 2 * n);
    for (int a = 0; a < m; ++a)
        for (int r = 0; r < n; ++r) {
            double re = qr[(size_t)r * m + a], im = qi[(size_t)r * m + a];
            qah[(size_t)a * 2 * n + r] = re;
            qah[(size_t)a * 2 * n + n + r] = im;
            qah[(size_t)(m + a) * 2 * n + r] = -im;
            qah[(size_t)(m + a) * 2 * n + n + r] = re;
        }
    upload(c, c->d_qap, qap);
    upload(c, c->d_qah, qah);
    // GEMM3 B per component: [(plane,q)][(plane',k)] = [[QAr, QAi], [-QAi, QAr]]
    for (int comp = 0; comp < 2; ++comp) {
        int nc = P.ncomp[comp], off = P.comp_off[comp];
        std::vector<double> q3((size_t)2 * nc * 2 * m);
        for (int q = 0; q < nc; ++q)
            for (int k = 0; k < m; ++k) {
                double re = qr[(size_t)(off + q) * m + k], im = qi[(size_t)(off + q) * m + k];
                q3[(size_t)q * 2 * m + k] = re;
                q3[(size_t)q * 2 * m + m + k] = im;
                q3[(size_t)(nc + q) * 2 * m + k] = -im;
                q3[(size_t)(nc + q) * 2 * m + m + k] = re;
            }
        upload(c, c->d_qar[comp], q3);
    }
    if (c->cfg.breit) {
        // QB of the internal (Kramers-sorted) spinors from QA: QB(j) =
        // -conj(QA(jbar)) for unbarred j, QB(jbar) = conj(QA(j))
        // (kramers.F:134-150)
        std::vector<double> br((size_t)n * m), bi((size_t)n * m);
        for (int i = 0; i < m; ++i) {
            const int t = c->itrmo[i], pi = std::abs(t) - 1;
            const double sg = t > 0 ? -1.0 : 1.0;
            for (int r = 0; r < n; ++r) {
                br[(size_t)r * m + i] = sg * qr[(size_t)r * m + pi];
                bi[(size_t)r * m + i] = -sg * qi[(size_t)r * m + pi];
            }
        }
        std::vector<double> qbh((size_t)2 * m * 2 * n), qbhs((size_t)2 * m * 2 * n, 0.0);
        for (int a = 0; a < m; ++a)
            for (int r = 0; r < n; ++r) {
                double re = br[(size_t)r * m + a], im = bi[(size_t)r * m + a];
                qbh[(size_t)a * 2 * n + r] = re;
                qbh[(size_t)a * 2 * n + n + r] = im;
                qbh[(size_t)(m + a) * 2 * n + r] = -im;
                qbh[(size_t)(m + a) * 2 * n + n + r] = re;
                if (r >= P.nL)  // small-component rows only (trans1.F:91-96 reads HA's S rows)
                    for (int x : {a * 2 * n + r, a * 2 * n + n + r, (m + a) * 2 * n + r, (m + a) * 2 * n + n + r})
                        qbhs[(size_t)x] = qbh[(size_t)x];
            }
        upload(c, c->d_qbh, qbh);
        upload(c, c->d_qbhS, qbhs);
        for (int comp = 0; comp < 2; ++comp) {
            int nc = P.ncomp[comp], off = P.comp_off[comp];
            std::vector<double> q3((size_t)2 * nc * 2 * m);
            for (int q = 0; q < nc; ++q)
                for (int k = 0; k < m; ++k) {
                    double re = br[(size_t)(off + q) * m + k], im = bi[(size_t)(off + q) * m + k];
                    q3[(size_t)q * 2 * m + k] = re;
                    q3[(size_t)q * 2 * m + m + k] = im;
                    q3[(size_t)(nc + q) * 2 * m + k] = -im;
                    q3[(size_t)(nc + q) * 2 * m + m + k] = re;
                }
            upload(c, c->d_qbr[comp], q3);
        }
    }
    // split path: slice the constant operands once
    if (c->cfg.precision == RT_PREC_SPLIT_BF16) split_prepare_constants(c);
}

// items of TRANS2's loop (trans2.F:73-74,230-239), records, screening data
static void plan_items(rt_ctx* c) {
    Plan& P = c->plan;
    Work& w = W(c);
    const int m = P.m, K = P.K;
    P.items.clear();
    // TRANS2's loops over the caller's spinor numbers (trans2.F:230-239) set
    // the record order; the items hold internal spinor indices
    std::vector<int> u2i(m);
    for (int i = 0; i < m; ++i) u2i[c->spin_user[i]] = i;
    for (int Iu = 0; Iu < m; ++Iu) {
        const int I = u2i[Iu];
        int ikr = c->ikrmo[I];
        if (ikr > 0) continue;  // records are written for barred I only
        for (int Ju = 0; Ju < m; ++Ju) {
            const int J = u2i[Ju];
            int jkr = c->ikrmo[J];
            if (std::abs(jkr) > std::abs(ikr)) continue;
            P.items.push_back({I, J, std::abs(ikr), std::abs(jkr), jkr < 0 ? 1 : 0});
        }
    }
    w.items4.resize(P.items.size());
    w.isign.resize(P.items.size());
    for (size_t t = 0; t < P.items.size(); ++t) {
        const Item& it = P.items[t];
        int ib = std::abs(c->itrmo[it.I]) - 1, jb = std::abs(c->itrmo[it.J]) - 1;
        w.items4[t] = make_int4(it.I, it.J, ib, jb);
        w.isign[t] = ((c->itrmo[it.I] > 0) == (c->itrmo[it.J] > 0)) ? 1.0f : -1.0f;
    }
    // records: class streams in item order
    w.recs.clear();
    w.item_rec0.assign(P.items.size() + 1, 0);
    for (int cc = 0; cc < 4; ++cc) { w.cap[cc] = 0; w.nrec[cc] = 0; }
    const bool all = c->cfg.throut < 0.0;
    for (size_t t = 0; t < P.items.size(); ++t) {
        const Item& it = P.items[t];
        w.item_rec0[t] = (int)w.recs.size();
        for (int cc = it.cls1 ? 0 : 1; cc <= (it.cls1 ? 0 : 3); ++cc) {
            EmitRec r;
            r.ijl = 0;  // filled per chunk
            r.cls = cc;
            r.ikr = it.ikr;
            r.jkr = it.jkr;
            r.rank = (int)w.nrec[cc]++;
            w.cap[cc] += set_size(cc, it.ikr, it.jkr, K, all);
            w.recs.push_back(r);
        }
    }
    w.item_rec0[P.items.size()] = (int)w.recs.size();
    // VMX (getmos.F:229-235) and the pair screening products
    std::vector<double> vmx(P.n, 0.0);
    for (int p = 0; p < P.n; ++p)
        for (int i = 0; i < m; ++i) {
            double re = c->qa[2 * ((size_t)p + (size_t)i * P.n)], im = c->qa[2 * ((size_t)p + (size_t)i * P.n) + 1];
            vmx[p] = std::max(vmx[p], std::hypot(re, im));
        }
    w.pair_vmx.resize(P.P);
    for (int i = 0; i < P.P; ++i) w.pair_vmx[i] = vmx[P.pair_p[i]] * vmx[P.pair_q[i]];
}

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
#define API_TRY try {
#define API_CATCH                                                     \
    }                                                                 \
    catch (const rt::Error& e) {                                      \
        ctx->err = e.msg;                                             \
        return e.code;                                                \
    }                                                                 \
    catch (const std::bad_alloc&) {                                   \
        ctx->err = "host allocation failed";                          \
        return RT_ERR_PROGRAM;                                        \
    }                                                                 \
    catch (const std::exception& e) {                                 \
        ctx->err = e.what();                                          \
        return RT_ERR_PROGRAM;                                        \
    }                                                                 \
    return RT_OK;

static thread_local std::string g_create_err;
static const char* const UNUSABLE_MSG =
    "context unusable: an aborted GEMM could not confirm that its tensor-core work and copies had finished";

void rt::set_thread_error(const std::string& msg) { g_create_err = msg; }

extern "C" int rt_create(rt_ctx** out, const rt_config* cfg) {
    if (!out) return RT_ERR_USER;
    *out = nullptr;
    rt_ctx* ctx = new (std::nothrow) rt_ctx();
    if (!ctx) return RT_ERR_PROGRAM;
    API_TRY
    check_config(cfg);
    ctx->cfg = *cfg;
    if (cfg->n_irrep == 4) ctx->ao_irrep.assign(cfg->ao_irrep, cfg->ao_irrep + cfg->nsc);
    ctx->cfg.ao_irrep = nullptr;
    if (ctx->cfg.slices == 0) ctx->cfg.slices = 5;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        throw Error(RT_ERR_PROGRAM, "no CUDA device: the library has no CPU path");
    }
    RT_CUDA(cudaGetDevice(&ctx->device));
    cudaDeviceProp prop;
    RT_CUDA(cudaGetDeviceProperties(&prop, ctx->device));
    if (prop.major != 10 || prop.minor != 3)
        throw Error(RT_ERR_PROGRAM, std::string("the library is built for sm_103a; device is ") +
                                        prop.name);
    RT_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    for (auto& e : ctx->ev) RT_CUDA(cudaEventCreate(&e));
    const char* trace = std::getenv("RT_TRACE");
    ctx->trace.on = trace && *trace && std::strcmp(trace, "0") != 0;
    plan_ao(ctx);
    *out = ctx;
    return RT_OK;
    }
    catch (const rt::Error& e) {
        g_create_err = e.msg;
        rt_destroy(ctx);
        return e.code;
    }
    catch (...) {
        g_create_err = "rt_create failed";
        rt_destroy(ctx);
        return RT_ERR_PROGRAM;
    }
}

extern "C" int rt_set_coefficients(rt_ctx* ctx, const double* qa, int ld_qa, const int* itrmo,
                                   const int* kra, const int* krb, const int* ikrmo,
                                   const int* imoras_pairs) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    const int n = ctx->plan.n, m = ctx->plan.m, K = ctx->plan.K;
    if (!qa || !itrmo || !kra || !krb || !ikrmo) throw Error(RT_ERR_USER, "null coefficient table");
    if (ld_qa < n) throw Error(RT_ERR_USER, "ld_qa < NSC");
    // consistency of the Kramers tables (getmos.F:166-199, kramers.F:114-115)
    for (int i = 0; i < m; ++i) {
        int j = std::abs(itrmo[i]);
        if (j < 1 || j > m || j == i + 1 || itrmo[j - 1] != -(itrmo[i] > 0 ? 1 : -1) * (i + 1))
            throw Error(RT_ERR_PROGRAM, "ITRMO does not pair the spinors (Kramers symmetry error)");
    }
    for (int k = 0; k < K; ++k) {
        int a = kra[k], b = krb[k];
        if (a < 1 || a > m || b < 1 || b > m || itrmo[a - 1] != b || ikrmo[a - 1] != k + 1 ||
            ikrmo[b - 1] != -(k + 1))
            throw Error(RT_ERR_PROGRAM, "KRA/KRB/IKRMO inconsistent with ITRMO");
    }
    // Internal spinor order: the unbarred members KRA(1..K), then the barred
    // members KRB(1..K).  All device work runs in this Kramers-sorted basis;
    // MDCINT labels are Kramers indices and do not depend on it.
    ctx->spin_user.assign(m, 0);
    for (int q = 0; q < K; ++q) {
        ctx->spin_user[q] = kra[q] - 1;
        ctx->spin_user[K + q] = krb[q] - 1;
    }
    ctx->qa.assign((size_t)2 * n * m, 0.0);
    for (int i = 0; i < m; ++i)
        std::memcpy(&ctx->qa[(size_t)2 * i * n], qa + (size_t)2 * ctx->spin_user[i] * ld_qa,
                    sizeof(double) * 2 * n);
    for (double v : ctx->qa)
        if (!std::isfinite(v)) throw Error(RT_ERR_USER, "non-finite spinor coefficient");
    ctx->itrmo.assign(m, 0);
    ctx->ikrmo.assign(m, 0);
    ctx->kra.assign(K, 0);
    ctx->krb.assign(K, 0);
    for (int q = 0; q < K; ++q) {
        ctx->itrmo[q] = K + q + 1;   // ITRMO(KRA) = +KRB
        ctx->itrmo[K + q] = -(q + 1);  // ITRMO(KRB) = -KRA
        ctx->ikrmo[q] = q + 1;
        ctx->ikrmo[K + q] = -(q + 1);
        ctx->kra[q] = q + 1;
        ctx->krb[q] = K + q + 1;
    }
    ctx->imoras.assign(2 * K, 0);
    if (imoras_pairs) ctx->imoras.assign(imoras_pairs, imoras_pairs + 2 * K);
    else
        for (int k = 0; k < K; ++k) { ctx->imoras[2 * k] = kra[k]; ctx->imoras[2 * k + 1] = krb[k]; }
    plan_items(ctx);
    build_coef_device(ctx);
    RT_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->have_coef = true;
    ++ctx->gen;
    API_CATCH
}

// grow the device record store to hold `need` integrals
static void ensure_record_capacity(rt_ctx* c, long long need) {
    if (need <= c->cap_int) return;
    long long cap = std::max(need, c->cap_int * 2);
    double* v = dalloc<double>(c, cap);
    int* a = dalloc<int>(c, cap);
    int* b = dalloc<int>(c, cap);
    if (c->n_int > 0) {
        RT_CUDA(cudaMemcpyAsync(v, c->d_rint, c->n_int * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        RT_CUDA(cudaMemcpyAsync(a, c->d_l2, c->n_int * sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
        RT_CUDA(cudaMemcpyAsync(b, c->d_l1, c->n_int * sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
        RT_CUDA(cudaStreamSynchronize(c->stream));
    }
    dfree(c, c->d_rint);
    dfree(c, c->d_l2);
    dfree(c, c->d_l1);
    c->d_rint = v;
    c->d_l2 = a;
    c->d_l1 = b;
    c->cap_int = cap;
}

static void flush_staged(rt_ctx* c) {
    long long ns = (long long)c->st_v.size();
    if (ns == 0) return;
    ensure_record_capacity(c, c->n_int + ns);
    RT_CUDA(cudaMemcpyAsync(c->d_rint + c->n_int, c->st_v.data(), ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    RT_CUDA(cudaMemcpyAsync(c->d_l2 + c->n_int, c->st_l2.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    RT_CUDA(cudaMemcpyAsync(c->d_l1 + c->n_int, c->st_l1.data(), ns * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    RT_CUDA(cudaStreamSynchronize(c->stream));
    c->n_int += ns;
    c->st_v.clear();
    c->st_l2.clear();
    c->st_l1.clear();
}

// Copy of `bytes` split over the context's copy streams (created on first
// use); sync_pieces waits for all of them.
static void copy_pieces(rt_ctx* c, void* dst, const void* src, size_t bytes) {
    const int ns = (int)(sizeof(c->cstream) / sizeof(c->cstream[0]));
    if (!c->cstream[0])
        for (int i = 0; i < ns; ++i) RT_CUDA(cudaStreamCreateWithFlags(&c->cstream[i], cudaStreamNonBlocking));
    const size_t piece = std::max<size_t>((size_t)64 << 20, (bytes + ns - 1) / ns);
    int i = 0;
    for (size_t o = 0; o < bytes; o += piece, ++i)
        RT_CUDA(cudaMemcpyAsync((char*)dst + o, (const char*)src + o, std::min(piece, bytes - o),
                                cudaMemcpyDefault, c->cstream[i % ns]));
}

static void sync_pieces(rt_ctx* c) {
    for (auto s : c->cstream)
        if (s) RT_CUDA(cudaStreamSynchronize(s));
}

// ---- the queued next record set (rt_queue_ao_records_bulk) ----
// Its copies go into the record arrays at offset 0 on the prefetch streams,
// which only rt_transform issues while it runs (after its bucketing, the last
// reader of the current records); every other call that touches the records
// applies the queue first.
static void rq_issue(rt_ctx* c) {
    auto& q = c->rq;
    if (!q.pending || q.issued) return;
    const int ns = (int)(sizeof(c->pstream) / sizeof(c->pstream[0]));
    if (!c->pstream[0])
        for (int i = 0; i < ns; ++i) RT_CUDA(cudaStreamCreateWithFlags(&c->pstream[i], cudaStreamNonBlocking));
    if (q.tot > c->cap_int) throw Error(RT_ERR_INTERNAL, "queued records exceed the record arrays");
    auto pieces = [&](void* dst, const void* src, size_t bytes, int& k) {
        const size_t piece = std::max<size_t>((size_t)64 << 20, (bytes + ns - 1) / ns);
        for (size_t o = 0; o < bytes; o += piece, ++k)
            RT_CUDA(cudaMemcpyAsync((char*)dst + o, (const char*)src + o, std::min(piece, bytes - o),
                                    cudaMemcpyDefault, c->pstream[k % ns]));
    };
    int k = 0;
    if (q.tot > 0) {
        pieces(c->d_rint, q.rint, q.tot * sizeof(double), k);
        pieces(c->d_l2, q.l2, q.tot * sizeof(int), k);
        pieces(c->d_l1, q.l1, q.tot * sizeof(int), k);
    }
    q.issued = true;
}

// Wait for the queued copies and make the queued set the context's records.
// Returns the first CUDA error of the wait (the records are then undefined).
static cudaError_t rq_finish(rt_ctx* c) noexcept {
    auto& q = c->rq;
    if (!q.pending) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    for (auto s : c->pstream)
        if (s) {
            const cudaError_t x = cudaStreamSynchronize(s);
            if (e == cudaSuccess) e = x;
        }
    c->rec_file = std::move(q.file);
    c->rec_it = std::move(q.it);
    c->rec_nt = std::move(q.nt);
    c->rec_off.resize(c->rec_nt.size());
    long long off = 0;
    for (size_t r = 0; r < c->rec_nt.size(); ++r) {
        c->rec_off[r] = off;
        off += c->rec_nt[r];
    }
    c->n_int = q.tot;
    q = rt_ctx::RecordQueue();
    ++c->gen;
    return e;
}

// Any call other than rt_transform that reads or changes the records
// applies a queued set first, synchronously.
static void rq_apply(rt_ctx* c) {
    if (!c->rq.pending) return;
    rq_issue(c);
    const cudaError_t e = rq_finish(c);
    if (e != cudaSuccess) throw Error(RT_ERR_PROGRAM, std::string("queued record copies: ") + cudaGetErrorString(e));
}

// The host copies of an earlier transform's elements (deferred mode)
// complete before anything rewrites or hands out its results.
static void host_result_wait(rt_ctx* c) {
    if (!c->host_inflight) return;
    c->host_inflight = false;
    RT_CUDA(cudaStreamSynchronize(c->cstream[0]));
}

static void add_record_meta(rt_ctx* c, int file, int it, long long nt, long long off) {
    c->rec_file.push_back(file);
    c->rec_it.push_back(it);
    c->rec_nt.push_back(nt);
    c->rec_off.push_back(off);
}

extern "C" int rt_add_ao_records(rt_ctx* ctx, int file_class, int nt, int itype, const double* rint,
                                 const int* label2, const int* label1) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    if (nt < 0) throw Error(RT_ERR_USER, "negative record length");
    if (file_class < 1 || file_class > 4) throw Error(RT_ERR_USER, "file class must be 1..4");
    if (nt > 0 && (!rint || !label2 || !label1)) throw Error(RT_ERR_USER, "null record arrays");
    rq_apply(ctx);
    long long off = ctx->n_int + (long long)ctx->st_v.size();
    add_record_meta(ctx, file_class, itype, nt, off);
    ctx->st_v.insert(ctx->st_v.end(), rint, rint + nt);
    ctx->st_l2.insert(ctx->st_l2.end(), label2, label2 + nt);
    ctx->st_l1.insert(ctx->st_l1.end(), label1, label1 + nt);
    if (ctx->st_v.size() >= (size_t)(8 << 20)) flush_staged(ctx);
    ctx->transformed = false;
    ++ctx->gen;
    API_CATCH
}

extern "C" int rt_add_ao_records_bulk(rt_ctx* ctx, long long nrec, const int* file_class,
                                      const long long* nt, const int* itype, const double* rint,
                                      const int* label2, const int* label1) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    if (nrec < 0) throw Error(RT_ERR_USER, "negative record count");
    long long tot = 0;
    for (long long r = 0; r < nrec; ++r) {
        if (nt[r] < 0) throw Error(RT_ERR_USER, "negative record length");
        if (file_class[r] < 1 || file_class[r] > 4) throw Error(RT_ERR_USER, "file class must be 1..4");
        tot += nt[r];
    }
    rq_apply(ctx);
    flush_staged(ctx);
    long long off = ctx->n_int;
    for (long long r = 0; r < nrec; ++r) {
        add_record_meta(ctx, file_class[r], itype[r], nt[r], off);
        off += nt[r];
    }
    ensure_record_capacity(ctx, ctx->n_int + tot);
    if (tot > 0) {
        // large transfers in pieces on several streams (several copy engines)
        copy_pieces(ctx, ctx->d_rint + ctx->n_int, rint, tot * sizeof(double));
        copy_pieces(ctx, ctx->d_l2 + ctx->n_int, label2, tot * sizeof(int));
        copy_pieces(ctx, ctx->d_l1 + ctx->n_int, label1, tot * sizeof(int));
        sync_pieces(ctx);
    }
    ctx->n_int += tot;
    ctx->transformed = false;
    ++ctx->gen;
    API_CATCH
}

extern "C" int rt_queue_ao_records_bulk(rt_ctx* ctx, long long nrec, const int* file_class,
                                       const long long* nt, const int* itype, const double* rint,
                                       const int* label2, const int* label1) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    if (nrec < 0) throw Error(RT_ERR_USER, "negative record count");
    if (nrec > 0 && (!file_class || !nt || !itype)) throw Error(RT_ERR_USER, "null record tables");
    long long tot = 0;
    for (long long r = 0; r < nrec; ++r) {
        if (nt[r] < 0) throw Error(RT_ERR_USER, "negative record length");
        if (file_class[r] < 1 || file_class[r] > 4) throw Error(RT_ERR_USER, "file class must be 1..4");
        tot += nt[r];
    }
    if (tot > 0 && (!rint || !label2 || !label1)) throw Error(RT_ERR_USER, "null record arrays");
    rq_apply(ctx);  // a set queued before and not yet transformed
    flush_staged(ctx);
    ensure_record_capacity(ctx, tot);  // keeps the current records
    auto& q = ctx->rq;
    q.file.assign(file_class, file_class + nrec);
    q.it.assign(itype, itype + nrec);
    q.nt.assign(nt, nt + nrec);
    q.tot = tot;
    q.rint = rint;
    q.l2 = label2;
    q.l1 = label1;
    q.issued = false;
    q.pending = true;
    API_CATCH
}

extern "C" int rt_clear_ao_records(rt_ctx* ctx) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    rq_apply(ctx);
    ctx->n_int = 0;
    ctx->st_v.clear();
    ctx->st_l2.clear();
    ctx->st_l1.clear();
    ctx->rec_file.clear();
    ctx->rec_it.clear();
    ctx->rec_nt.clear();
    ctx->rec_off.clear();
    ctx->transformed = false;
    ++ctx->gen;
    API_CATCH
}

// ---------------------------------------------------------------------------
// the transformation
// ---------------------------------------------------------------------------
namespace {

// rotran's half buckets (LABEL1 pair only) and the two-half record assembly:
// always for the Gaunt transform, on request for the Coulomb one
bool uses_halves(const rt_ctx* c) { return c->cfg.breit != 0 || c->cfg.half_buckets != 0; }

void ensure_fixed(rt_ctx* c, int& pair_chunk, int& item_chunk, bool exact = false) {
    Plan& P = c->plan;
    Work& w = W(c);
    const int n = P.n, m = P.m;
    const long long KK1 = (long long)P.items.size();
    const int S0 = c->cfg.precision == RT_PREC_SPLIT_BF16 ? c->cfg.slices : 0;
    plan_expand(c, S0);
    if (!c->d_bcount) {
        c->d_bcount = dalloc<int>(c, (size_t)P.P + 1);
        c->d_boff = dalloc<long long>(c, (size_t)P.P + 1);
    }
    if (!c->d_jstart || c->bucket_n != P.nbuckets) {
        dfree(c, c->d_jstart);
        dfree(c, c->d_jcount);
        c->d_jstart = dalloc<long long>(c, (size_t)std::max(1LL, P.nbuckets));
        c->d_jcount = dalloc<int>(c, (size_t)std::max(1LL, P.nbuckets));
        c->bucket_n = P.nbuckets;
    }
    // pq buckets: up to two entries per integral; (pq, job) buckets: four
    if (c->bucket_cap < 2 * c->n_int) {
        dfree(c, c->d_bval);
        dfree(c, c->d_brs);
        dfree(c, c->d_jval);
        dfree(c, c->d_jrs);
        c->bucket_cap = std::max(1LL, 2 * c->n_int);
        c->d_bval = dalloc<double>(c, (size_t)c->bucket_cap);
        c->d_brs = dalloc<int>(c, (size_t)c->bucket_cap);
        c->d_jval = dalloc<double>(c, (size_t)2 * c->bucket_cap);
        c->d_jrs = dalloc<int>(c, (size_t)2 * c->bucket_cap);
    }
    if (!c->d_hp) c->d_hp = dalloc<double>(c, (size_t)2 * KK1 * P.P * (c->cfg.breit ? 3 : 1));
    if (uses_halves(c) && !c->d_rl_all) c->d_rl_all = dalloc<double>(c, (size_t)2 * KK1 * m * m);
    for (int cc = 0; cc < 4; ++cc) {
        if (!c->d_oidx[cc]) {
            c->d_oidx[cc] = dalloc<int>(c, (size_t)2 * std::max(1LL, w.cap[cc]));
            c->d_oval[cc] = dalloc<double>(c, (size_t)2 * std::max(1LL, w.cap[cc]));
            c->d_hdr[cc] = dalloc<int>(c, (size_t)std::max(1LL, w.nrec[cc]));          // counts
            c->out_cap[cc] = w.cap[cc];
        }
    }
    // work arena from the memory budget
    size_t freeb = 0, totb = 0;
    RT_CUDA(cudaMemGetInfo(&freeb, &totb));
    // the work arena held from the previous call is given back before a
    // resize, so it counts as free (else chunks would shrink on every call)
    const size_t held = c->ha_len * sizeof(double) + split_work_bytes(c);
    long long budget = c->cfg.mem_budget > 0
                           ? c->cfg.mem_budget - (long long)c->dev_bytes + (long long)c->ha_len * 8
                           : (long long)(0.85 * (double)(freeb + held));
    const int S = c->cfg.precision == RT_PREC_SPLIT_BF16 ? c->cfg.slices : 0;
    // bytes per pair of stage A and per item of stage B
    long long a_pp = 0;
    for (long long v : P.pg_a_pp) a_pp = std::max(a_pp, v);
    const bool breit = c->cfg.breit != 0;
    // Gaunt: a second RI (QB^H HA) per pair; three RLR per item
    double per_pair = 16.0 * n * m + (breit ? 32.0 : 16.0) * m * m + (S ? 0.0 : 8.0 * a_pp);
    int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
    const double m3_el = breit ? (double)P.ncomp[0] * P.ncomp[1] : (double)ncmax * ncmax;
    double per_item = 16.0 * m3_el + 16.0 * n * m + (breit ? 48.0 : 16.0) * m * m;
    if (S) {
        per_pair += split_stageA_bytes_per_pair(c);
        per_item += split_stageB_bytes_per_item(c);
    }
    int maxpg = 1;
    for (auto& g : P.pgroups) maxpg = std::max(maxpg, g.size);
    long long usable = budget - (64LL << 20);
    if (usable <= 0) throw Error(RT_ERR_DIM, "device memory budget exhausted by the fixed arrays");
    pair_chunk = (int)std::min<long long>(maxpg, std::max(1LL, (long long)(usable / per_pair)));
    item_chunk = (int)std::min<long long>(KK1, std::max(1LL, (long long)(usable / per_item)));
    pair_chunk = std::min(pair_chunk, 16384);
    item_chunk = std::min(item_chunk, 16384);
    if (exact) {  // one chunk per pair group and one item chunk (batched transforms)
        pair_chunk = maxpg;
        item_chunk = (int)std::max(1LL, KK1);
        if ((double)usable < per_pair * pair_chunk || (double)usable < per_item * item_chunk)
            throw Error(RT_ERR_DIM, "device memory too small for a single-chunk (batched) transform");
    }
    if (usable < per_pair || usable < per_item)
        throw Error(RT_ERR_DIM, "device memory budget too small for one pair / one item");
    size_t need_a = (size_t)((per_pair - (S ? split_stageA_bytes_per_pair(c) : 0)) * pair_chunk / 8) + 64;
    size_t need_b = (size_t)((per_item - (S ? split_stageB_bytes_per_item(c) : 0)) * item_chunk / 8) + 64;
    size_t need = std::max(need_a, need_b);
    if (!c->d_ha || c->stage.pair_chunk != pair_chunk || c->stage.item_chunk != item_chunk) {
        // both old arenas go before either new one is allocated
        dfree(c, c->d_ha);
        c->d_ha = nullptr;
        c->ha_len = 0;
        c->stage.pair_chunk = c->stage.item_chunk = 0;
        if (S) split_alloc_work(c, pair_chunk, item_chunk);
        c->d_ha = dalloc<double>(c, need);
        c->ha_len = need;
        c->stage.pair_chunk = pair_chunk;
        c->stage.item_chunk = item_chunk;
    }
}

}  // namespace

static void upload_tables(rt_ctx* c, DeviceTabs& T, std::vector<void*>& tmp) {
    Plan& P = c->plan;
    auto up = [&](auto* hostp, size_t count, auto*& devp) {
        using TT = std::remove_const_t<std::remove_pointer_t<decltype(hostp)>>;
        TT* d = static_cast<TT*>(tmp_alloc(c, count * sizeof(TT)));
        if (count) RT_CUDA(cudaMemcpyAsync(d, hostp, count * sizeof(TT), cudaMemcpyHostToDevice, c->stream));
        devp = d;
        tmp.push_back(d);
    };
    const long long ntri = (long long)P.n * (P.n + 1) / 2;
    std::vector<unsigned char> pqr(ntri, 0);
    for (int p = 0; p < P.n; ++p)
        for (int q = 0; q <= p; ++q) {
            bool pl = p < P.nL, ql = q < P.nL;
            bool inc = c->cfg.breit ? pl != ql  // the SL blocks of the Gaunt integrals (makind.F:91-95)
                                    : !(!pl && ql) && !(!pl && c->cfg.mfil < 3);  // makind.F:75-77
            pqr[(long long)p * (p + 1) / 2 + q] = inc ? 1 : 0;
        }
    std::vector<int> pgroup(P.P), pgs, pgz, aopos(P.n), g1of(P.pgroups.size() * P.nblk, -1), g1k;
    for (size_t g = 0; g < P.pgroups.size(); ++g) {
        pgs.push_back(P.pgroups[g].start);
        pgz.push_back(P.pgroups[g].size);
        for (int i = 0; i < P.pgroups[g].size; ++i) pgroup[P.pgroups[g].start + i] = (int)g;
    }
    for (int p = 0; p < P.n; ++p) aopos[p] = P.ao_sorted[p] - P.blk_start[P.ao_block[p]];
    for (size_t g = 0; g < P.g1.size(); ++g) {
        g1of[P.g1[g].pg * P.nblk + P.g1[g].rblk] = (int)g;
        g1k.push_back(P.g1[g].kblk);
    }
    up(pqr.data(), pqr.size(), T.pq_read);
    up(P.pair_of_orig.data(), P.pair_of_orig.size(), T.pair_of_orig);
    up(pgroup.data(), pgroup.size(), T.pair_group);
    up(pgs.data(), pgs.size(), T.pg_start);
    up(pgz.data(), pgz.size(), T.pg_size);
    up(P.ao_block.data(), P.ao_block.size(), T.ao_block);
    up(aopos.data(), aopos.size(), T.ao_pos);
    up(P.blk_size.data(), P.blk_size.size(), T.blk_size);
    up(g1of.data(), g1of.size(), T.g1_of);
    up(g1k.data(), g1k.size(), T.g1_kblk);
    up(P.jb_base.data(), P.jb_base.size(), T.jb_base);
    up(P.jb_band.data(), P.jb_band.size(), T.jb_band);
    up(P.pg_njobs.data(), P.pg_njobs.size(), T.pg_njobs);
    up(P.pg_bbase.data(), P.pg_bbase.size(), T.pg_bbase);
}

namespace {

// Gaunt items: for TRANS2's item (I, J), UNIQUE with the Breit sign
// (unique.F:1-50; the sign is turned at unique.F:34) gives the pair JI whose
// values TRBOUT stored, and TROUT's enumeration of JI (IBAR, IK, JK >= IK:
// trbout.F:35-42) gives its spinors I' = KRA(IK) or KRB(IK), J' = KRB(JK).
std::vector<BreitItem> breit_items(rt_ctx* c) {
    const Plan& P = c->plan;
    const int K = P.K;
    std::vector<int2> ji_pair;  // JI-1 -> (I', J') internal, 0-based
    for (int ibar = 1; ibar <= 2; ++ibar)
        for (int ik = 1; ik <= K; ++ik)
            for (int jk = ik; jk <= K; ++jk)
                ji_pair.push_back(make_int2((ibar == 1 ? c->kra[ik - 1] : c->krb[ik - 1]) - 1, c->krb[jk - 1] - 1));
    std::vector<BreitItem> out(P.items.size());
    for (size_t t = 0; t < P.items.size(); ++t) {
        const Item& it = P.items[t];
        int ikr = c->ikrmo[it.I], jkr = c->ikrmo[it.J];
        int iikr, jjkr;
        bool conj;
        if (std::abs(ikr) >= std::abs(jkr)) { iikr = ikr; jjkr = jkr; conj = false; }
        else { iikr = jkr; jjkr = ikr; conj = true; }
        int is = 1;
        if (iikr > 0) {
            is = (iikr * jjkr >= 0) ? 1 : -1;
            is = -is;  // Breit
            iikr = -iikr;
            jjkr = -jjkr;
            conj = !conj;
        }
        const int off = K * (K + 1) / 2;
        const int ij = jjkr > 0 ? (jjkr - 1) * (2 * K - jjkr) / 2 - iikr : off - (jjkr + 1) * (2 * K + jjkr) / 2 - iikr;
        if (ij < 1 || ij > (int)ji_pair.size()) throw Error(RT_ERR_INTERNAL, "Gaunt item outside the JI list");
        const int I2 = ji_pair[ij - 1].x, J2 = ji_pair[ij - 1].y;
        BreitItem b;
        b.x = J2;
        b.y = I2;
        b.xb = std::abs(c->itrmo[J2]) - 1;
        b.yb = std::abs(c->itrmo[I2]) - 1;
        b.s = ((c->itrmo[J2] > 0) == (c->itrmo[I2] > 0)) ? -1.0f : 1.0f;
        b.conj = conj ? 1 : 0;
        b.neg = is < 0 ? 1 : 0;
        out[t] = b;
    }
    return out;
}

// Device tables and temporaries of one pass over the integral records
// (rt_transform and rt_adjoint), freed when the pass ends.
struct Pass {
    rt_ctx* c = nullptr;
    std::vector<void*> tmp;
    DeviceTabs T{};
    long long* d_roff = nullptr;
    int2* d_rmeta = nullptr;
    int4* d_items = nullptr;
    float* d_isign = nullptr;
    double* d_pvmx = nullptr;
    int *d_kra = nullptr, *d_krb = nullptr, *d_itrmo = nullptr;
    int* d_pidx[2] = {nullptr, nullptr};
    BreitItem* d_bitems = nullptr;  // Gaunt: UNIQUE's stored pair per item
    int* d_item_of = nullptr;       // Gaunt: item of Kramers (i, j), [J barred][i][j]
    unsigned long long* d_stat = nullptr;
    int pair_chunk = 0, item_chunk = 0;
    int launches = 0;
    bool split = false;
    explicit Pass(rt_ctx* ctx) : c(ctx) {}
    ~Pass() {
        // kernels of this pass may still be queued (an error path, or a batch
        // whose launches ran on other streams); pooled blocks must be idle
        tmp_release(c, tmp, cudaDeviceSynchronize() == cudaSuccess);
    }
    template <class T>
    T* alloc(size_t count) {
        T* p = static_cast<T*>(tmp_alloc(c, count * sizeof(T)));
        tmp.push_back(p);
        return p;
    }
    template <class T>
    T* upload(const T* host, size_t count) {
        T* p = alloc<T>(count);
        if (count) RT_CUDA(cudaMemcpyAsync(p, host, count * sizeof(T), cudaMemcpyHostToDevice, c->stream));
        return p;
    }
};

// Work arena, tables, item and Kramers tables on the device.
void pass_setup(Pass& ps, bool exact = false) {
    rt_ctx* ctx = ps.c;
    Plan& P = ctx->plan;
    Work& w = W(ctx);
    const int m = P.m, K = P.K;
    const int KK1 = (int)P.items.size();
    ps.split = ctx->cfg.precision == RT_PREC_SPLIT_BF16;
    ensure_fixed(ctx, ps.pair_chunk, ps.item_chunk, exact);
    upload_tables(ctx, ps.T, ps.tmp);
    std::vector<int2> meta(ctx->rec_off.size());
    for (size_t r = 0; r < meta.size(); ++r) meta[r] = make_int2(ctx->rec_file[r], ctx->rec_it[r]);
    ps.d_roff = ps.upload(ctx->rec_off.data(), ctx->rec_off.size());
    ps.d_rmeta = ps.upload(meta.data(), meta.size());
    ps.d_items = ps.upload(w.items4.data(), (size_t)KK1);
    ps.d_isign = ps.upload(w.isign.data(), (size_t)KK1);
    ps.d_pvmx = ps.upload(w.pair_vmx.data(), (size_t)P.P);
    ps.d_kra = ps.upload(ctx->kra.data(), (size_t)K);
    ps.d_krb = ps.upload(ctx->krb.data(), (size_t)K);
    ps.d_itrmo = ps.upload(ctx->itrmo.data(), (size_t)m);
    for (int cc = 0; cc < 2; ++cc) ps.d_pidx[cc] = ps.upload(P.pidx[cc].data(), P.pidx[cc].size());
    if (ctx->cfg.breit) {
        const std::vector<BreitItem> bi = breit_items(ctx);
        ps.d_bitems = ps.upload(bi.data(), bi.size());
    }
    if (uses_halves(ctx)) {
        std::vector<int> item_of((size_t)2 * K * K, -1);
        for (int t = 0; t < KK1; ++t) {
            const Item& it = P.items[t];
            item_of[((size_t)it.cls1 * K + it.ikr - 1) * K + it.jkr - 1] = t;
        }
        ps.d_item_of = ps.upload(item_of.data(), item_of.size());
    }
    ps.d_stat = ps.alloc<unsigned long long>(8);
    RT_CUDA(cudaMemsetAsync(ps.d_stat, 0, 8 * sizeof(unsigned long long), ctx->stream));
}

// THRGEN / VMX(p) VMX(q) per pair (+inf below THRGEN): the split path's
// FP32 screening threshold.
float* pass_pair_thr(Pass& ps, double thrgen) {
    const Work& w = W(ps.c);
    std::vector<float> t(w.pair_vmx.size());
    for (size_t i = 0; i < t.size(); ++i) {
        const double vv = w.pair_vmx[i];
        t[i] = vv < thrgen ? INFINITY : (float)(thrgen / vv);
    }
    return ps.upload(t.data(), t.size());
}

// Sort the records into pq buckets (SORT1) and check their labels.
void pass_bucketing(Pass& ps, bool halves) {
    rt_ctx* ctx = ps.c;
    Plan& P = ctx->plan;
    cudaStream_t st = ctx->stream;
    const DeviceTabs& T = ps.T;
    ScatterTabs tb{P.n, ctx->cfg.mfil, P.nblk, T.pq_read, T.pair_of_orig, T.pair_group, T.pg_start,
                   T.pg_size, T.ao_block, T.ao_pos, T.blk_size, T.g1_of, T.g1_kblk,
                   T.jb_base, T.jb_band, T.pg_bbase, T.pg_njobs};
    tb.breit = ctx->cfg.breit;
    tb.half = halves ? 1 : 0;
    launch_bucket(st, ctx->d_rint, ctx->d_l2, ctx->d_l1, ctx->n_int, ps.d_roff, ps.d_rmeta,
                  (int)ctx->rec_off.size(), tb, P.P, ctx->d_bcount, ctx->d_boff, ctx->d_bval,
                  ctx->d_brs, P.nbuckets, ctx->d_jstart, ctx->d_jcount, ctx->d_jval, ctx->d_jrs,
                  (unsigned int*)ps.d_stat);
    ps.launches += ctx->n_int > 0 ? 3 : 1;
    RT_CUDA(cudaGetLastError());
    ctx->trace.mark("bucketing kernels");
    unsigned long long hstat[8];
    RT_CUDA(cudaMemcpyAsync(hstat, ps.d_stat, sizeof(hstat), cudaMemcpyDeviceToHost, st));
    RT_CUDA(cudaStreamSynchronize(st));
    if (hstat[0] & ST_BAD_LABEL)
        throw Error(RT_ERR_USER, "integral label outside 1..NSC or pq label with q > p");
    if (hstat[0] & ST_BAD_BLOCK)
        throw Error(RT_ERR_USER, "integral outside the (LL|LL)/(SS|LL)/(SS|SS) or irrep block structure");
    RT_CUDA(cudaMemsetAsync(ps.d_stat, 0, 8 * sizeof(unsigned long long), st));
    ctx->trace.mark("bucketing status check");
}

// First half-transformation (TRANS1 + MTIMHER + TROUT) into the resident
// half-transformed array ctx->d_hp, one pair chunk at a time.
void pass_stage_a(Pass& ps, double thrgen) {
    rt_ctx* ctx = ps.c;
    Plan& P = ctx->plan;
    cudaStream_t st = ctx->stream;
    const int n = P.n, m = P.m;
    const int KK1 = (int)P.items.size();
    const bool split = ps.split;
    const int pair_chunk = ps.pair_chunk;
    KTimer& kt = ctx->ktimer;
    PhaseTrace& tr = ctx->trace;
    // the FP64 GEMMs are timed here; the split path times its tensor-core
    // kernels itself (rt_split.cu), without the slicing kernels around them
    auto gemm_begin = [&]() { if (!split) kt.begin(); };
    auto gemm_end = [&](double fl) { if (!split) kt.end(fl, fl); };
    // expansion jobs of every pair group
    std::vector<ExpandJob*> d_jobs(P.pgroups.size(), nullptr);
    for (size_t g = 0; g < P.pgroups.size(); ++g) {
        const auto& jv = P.pg_jobs[g];
        d_jobs[g] = ps.alloc<ExpandJob>(std::max<size_t>(1, jv.size()));
        if (!jv.empty())
            RT_CUDA(cudaMemcpyAsync(d_jobs[g], jv.data(), jv.size() * sizeof(ExpandJob), cudaMemcpyHostToDevice, st));
    }
    const int nsl = split ? ctx->cfg.slices : 0;
    float* d_pthr = pass_pair_thr(ps, thrgen);
    tr.mark("A: job and threshold tables");
    const bool breit = ctx->cfg.breit != 0;
    double* ha = ctx->d_ha;
    double* ri = ha + (size_t)2 * n * m * pair_chunk;
    double* ri2 = ri + (size_t)2 * m * m * pair_chunk;  // Gaunt: QB^H HA
    double* a1 = (breit ? ri2 : ri) + (size_t)2 * m * m * pair_chunk;  // FP64 GEMM1 operand (plain path)
    for (size_t g = 0; g < P.pgroups.size(); ++g) {
        const PairGroup& pg = P.pgroups[g];
        // does every r block meet this pair group?
        int covered = 0;
        size_t smem = 0;
        for (auto& gg : P.g1)
            if (gg.pg == (int)g) covered += P.blk_size[gg.rblk];
        for (auto& j : P.pg_jobs[g]) smem = std::max(smem, (size_t)(j.r_hi - j.r_lo) * j.nk * 8);
        for (int c0 = 0; c0 < pg.size; c0 += pair_chunk) {
            const int npc = std::min(pair_chunk, pg.size - c0);
            const long long plane = (long long)n * m * npc;
            if (covered < n) RT_CUDA(cudaMemsetAsync(ha, 0, 2 * plane * sizeof(double), st));
            // G_pq(r,s) of the chunk from the buckets
            if (!P.pg_jobs[g].empty()) {
                launch_expand_rows(st, nsl, ctx->d_jval, ctx->d_jrs, ctx->d_jstart, ctx->d_jcount, d_jobs[g],
                                   P.pg_njobs[g], P.pg_bbase[g] + (long long)c0 * P.pg_njobs[g], npc,
                                   smem, a1, split ? split_a1_slices(ctx) : nullptr,
                                   split ? split_a1_exps(ctx) : nullptr);
                ++ps.launches;
            }
            tr.mark("A: expand G_pq(r,s)");
            for (auto& gg : P.g1) {
                if (gg.pg != (int)g) continue;
                const int nr = P.blk_size[gg.rblk], nk = P.blk_size[gg.kblk];
                EpiHA epi{ha, P.blk_start[gg.rblk], m, npc, plane};
                gemm_begin();
                if (split)
                    split_gemm1(ctx, gg, npc, epi, &ps.launches);
                else
                    gemm_f64(st, a1 + gg.a_pp * npc, nk, (long long)npc * nk,
                             ctx->d_qap + (long long)P.blk_start[gg.kblk] * 2 * m, 2 * m, 0, npc, 2 * m, nk,
                             nr, epi), ++ps.launches;
                gemm_end(2.0 * npc * 2.0 * m * nk * nr);
            }
            tr.mark("A: GEMM1");
            EpiRowMajor e2{ri, (long long)m * npc, 0};
            if (breit) {
                // Gaunt (trans1.F:81-100): RIA = QA^H HA, RI2 = QB^H HA (S rows),
                // then TRBOUT's three streams for every item
                EpiRowMajor e2b{ri2, (long long)m * npc, 0};
                gemm_begin();
                if (split)
                    split_gemm2_breit(ctx, ha, 2 * n, (long long)m * npc, e2, e2b, &ps.launches);
                else {
                    gemm_f64(st, ctx->d_qah, 2 * n, 0, ha, (long long)m * npc, 0, 2 * m, m * npc, 2 * n, 1, e2);
                    gemm_f64(st, ctx->d_qbhS, 2 * n, 0, ha, (long long)m * npc, 0, 2 * m, m * npc, 2 * n, 1, e2b);
                    ps.launches += 2;
                }
                gemm_end(2.0 * 2.0 * 2 * m * (double)m * npc * 2 * n);
                tr.mark("A: slice HA + GEMM2 (QA and QB)");
                launch_trb_select(st, split, ri, ri2, m, npc, pg.start + c0, P.P, ps.d_bitems, KK1, ctx->d_hp,
                                  ps.d_stat + 1);
                ps.launches += (KK1 + 65534) / 65535;
                tr.mark("A: Gaunt selection");
                continue;
            }
            gemm_begin();
            if (split)
                split_gemm2_kramers(ctx, ha, 2 * n, (long long)m * npc, e2, &ps.launches);
            else
                gemm_f64(st, ctx->d_qah, 2 * n, 0, ha, (long long)m * npc, 0, 2 * m, m * npc, 2 * n, 1, e2), ++ps.launches;
            gemm_end(2.0 * 2 * m * (double)m * npc * 2 * n);
            tr.mark("A: slice HA + GEMM2");
            launch_tr_select(st, split, ri, m, npc, pg.start + c0, P.P, ps.d_items, ps.d_isign, KK1,
                             ps.d_pvmx, d_pthr, thrgen, ctx->d_hp, ps.d_stat + 1);
            ps.launches += (KK1 + 65534) / 65535;
            tr.mark("A: Kramers selection");
        }
    }
    RT_CUDA(cudaGetLastError());
}

// Algorithmic FLOPs of the transformation (dense-block count of the
// reference algorithm).
double algorithmic_flops(const Plan& P, double KK1, bool breit) {
    const int n = P.n, m = P.m;
    double f1 = 0.0;
    for (auto& gg : P.g1)
        f1 += 2.0 * P.blk_size[gg.rblk] * (double)P.pgroups[gg.pg].size * P.blk_size[gg.kblk] * 2.0 * m;
    // Gaunt: the second ZGEMM with QB (trans1.F:91-96)
    f1 += (breit ? 2.0 : 1.0) * (double)P.P * 8.0 * n * (double)m * m;
    double f2 = 0.0;
    if (breit)  // three streams, each MATMUL3/7 across the components and a ZGEMM
        f2 = KK1 * 3.0 * (2.0 * 8.0 * (double)P.ncomp[0] * P.ncomp[1] * m + 8.0 * n * (double)m * m);
    else {
        for (int cc = 0; cc < 2; ++cc) f2 += 8.0 * (double)P.ncomp[cc] * P.ncomp[cc] * m;
        f2 = KK1 * (f2 + 8.0 * n * (double)m * m);
    }
    return f1 + f2;
}

double algorithmic_flops(const Plan& P, bool breit) { return algorithmic_flops(P, (double)P.items.size(), breit); }

}  // namespace

extern "C" int rt_transform(rt_ctx* ctx) {
    if (!ctx) return RT_ERR_USER;
    // a queued record set becomes the context's records when this call
    // returns, whatever its outcome (its copies start after the bucketing)
    struct QueueGuard {
        rt_ctx* c;
        ~QueueGuard() {
            if (!c->rq.pending) return;
            // a call that ended early may still have bucketing kernels
            // reading the current records: they finish before the copies
            if (!c->rq.issued && cudaStreamSynchronize(c->stream) != cudaSuccess) c->unusable = true;
            try {
                rq_issue(c);
            } catch (...) {
            }
            if (rq_finish(c) != cudaSuccess) c->unusable = true;
        }
    } queue_guard{ctx};
    API_TRY
    if (ctx->unusable) throw Error(RT_ERR_PROGRAM, UNUSABLE_MSG);
    if (!ctx->have_coef) throw Error(RT_ERR_USER, "rt_set_coefficients has not been called");
    // the result arrays are rewritten from here on: an earlier result is
    // gone, and a transform that fails leaves none
    ctx->transformed = false;
    Plan& P = ctx->plan;
    Work& w = W(ctx);
    cudaStream_t st = ctx->stream;
    const int n = P.n, m = P.m, K = P.K;
    const int KK1 = (int)P.items.size();
    KTimer& kt = ctx->ktimer;
    kt.reset(st);
    PhaseTrace& tr = ctx->trace;
    tr.reset(st);
    tr.mark("start");
    RT_CUDA(cudaEventRecord(ctx->ev[0], st));
    flush_staged(ctx);
    RT_CUDA(cudaEventRecord(ctx->ev[1], st));
    tr.mark("staged records");
    Pass ps(ctx);
    pass_setup(ps);
    tr.mark("tables and work arena");
    const bool split = ps.split;
    auto gemm_begin = [&]() { if (!split) kt.begin(); };
    auto gemm_end = [&](double fl) { if (!split) kt.end(fl, fl); };
    // with result buffers on the host, stage B runs in at least four item
    // chunks so that each chunk's copy overlaps the following chunks' work
    const bool to_host = ctx->host_on;
    const int item_chunk = to_host ? std::min(ps.item_chunk, std::max(1, (KK1 + 3) / 4)) : ps.item_chunk;
    long long* d_total = ps.alloc<long long>(4);
    RT_CUDA(cudaMemsetAsync(d_total, 0, 4 * sizeof(long long), st));
    long long* d_off[4];
    for (int cc = 0; cc < 4; ++cc) d_off[cc] = ps.alloc<long long>(std::max(1LL, w.nrec[cc]));
    // ---- sort the records into pq buckets (SORT1) ----
    pass_bucketing(ps, uses_halves(ctx));
    RT_CUDA(cudaEventRecord(ctx->ev[2], st));
    if (ctx->rq.pending) {  // the raw records are read no more: the next set's copies overlap the rest
        rq_issue(ctx);
        tr.mark("next records queued");
    }
    // ---- stage A: first half-transformation (TRANS1) per pair chunk ----
    pass_stage_a(ps, ctx->cfg.thrgen);
    RT_CUDA(cudaEventRecord(ctx->ev[3], st));
    tr.mark("stage A tail");
    // ---- stage B: second half-transformation (TRANS2) + PPSYM per item chunk ----
    host_result_wait(ctx);  // the previous transform's copies (they overlapped stage A)
    double* m3 = ctx->d_ha;
    int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
    const bool breit = ctx->cfg.breit != 0, halves = uses_halves(ctx);
    const size_t m3_el = breit ? (size_t)P.ncomp[0] * P.ncomp[1] : (size_t)ncmax * ncmax;
    double* rk = m3 + 2 * m3_el * item_chunk;
    double* rlr = rk + (size_t)2 * n * m * item_chunk;
    double* rlr_b = rlr + (size_t)2 * m * m * item_chunk;   // Gaunt streams 2 and 3
    double* rlr_c = rlr_b + (size_t)2 * m * m * item_chunk;
    EmitRec* d_recs = ps.alloc<EmitRec>((size_t)3 * item_chunk);
    OutStreams os;
    for (int cc = 0; cc < 4; ++cc) {
        os.cnt[cc] = ctx->d_hdr[cc];
        os.off[cc] = d_off[cc];
        os.idx[cc] = ctx->d_oidx[cc];
        os.val[cc] = ctx->d_oval[cc];
    }
    os.total = d_total;
    std::vector<EmitRec> chunk_recs;
    // the elements of finished chunks to the caller's host buffers, on a copy
    // stream, while the next chunks run (the host has synchronised st)
    long long streamed[4] = {0, 0, 0, 0};
    if (to_host && !ctx->cstream[0]) RT_CUDA(cudaStreamCreateWithFlags(&ctx->cstream[0], cudaStreamNonBlocking));
    auto stream_out = [&]() {
        if (!to_host) return;
        long long tot[4];
        RT_CUDA(cudaMemcpy(tot, d_total, sizeof(tot), cudaMemcpyDeviceToHost));
        for (int c = 0; c < 4; ++c)
            if (tot[c] > ctx->host_cap[c]) {
                cudaStreamSynchronize(ctx->cstream[0]);   // no copy left in flight
                throw Error(RT_ERR_DIM, "rt_set_result_host: class " + std::to_string(c + 1) + " needs " +
                                            std::to_string(tot[c]) + " elements");
            }
        for (int c = 0; c < 4; ++c) {
            const long long a = streamed[c], nz = tot[c] - a;
            if (nz <= 0) continue;
            RT_CUDA(cudaMemcpyAsync(ctx->host_idx[c] + 2 * a, ctx->d_oidx[c] + 2 * a, 2 * nz * sizeof(int),
                                    cudaMemcpyDeviceToHost, ctx->cstream[0]));
            RT_CUDA(cudaMemcpyAsync(ctx->host_val[c] + 2 * a, ctx->d_oval[c] + 2 * a, 2 * nz * sizeof(double),
                                    cudaMemcpyDeviceToHost, ctx->cstream[0]));
            streamed[c] = tot[c];
        }
    };
    for (int i0 = 0; i0 < KK1; i0 += item_chunk) {
        const int nij = std::min(item_chunk, KK1 - i0);
        const long long rkplane = (long long)n * nij * m;
        // Gaunt (trans2.F:129-177): stream 1 MATMUL3 with QA then QA^H,
        // stream 2 MATMUL7 (x2) with QB then QA^H, stream 3 MATMUL7 (x2)
        // with QA then QB^H; rows of one component meet the other one's
        for (int sx = 0; breit && sx < 3; ++sx) {
            const double* hps = ctx->d_hp + (size_t)sx * 2 * KK1 * P.P;
            for (int rc = 0; rc < 2; ++rc) {
                const int oc = 1 - rc, nrow = P.ncomp[rc], ncol = P.ncomp[oc];
                if (nrow == 0 || ncol == 0) continue;
                launch_expand(st, hps, P.P, KK1, i0, nij, ps.d_pidx[rc], nrow, ncol, m3, sx > 0, split);
                ++ps.launches;
                EpiRK e3{rk, m, (long long)P.comp_off[rc] * nij, rkplane};
                gemm_begin();
                if (split)
                    split_gemm3_op(ctx, sx == 1 ? 1 : 0, oc, m3, nrow, ncol, nij, e3, &ps.launches);
                else
                    gemm_f64(st, m3, 2 * ncol, 0, sx == 1 ? ctx->d_qbr[oc] : ctx->d_qar[oc], 2 * m, 0, nrow * nij,
                             2 * m, 2 * ncol, 1, e3), ++ps.launches;
                gemm_end(2.0 * nrow * (double)nij * 2 * m * 2 * ncol);
            }
            tr.mark("B: Gaunt expand + GEMM3");
            double* out = sx == 0 ? rlr : sx == 1 ? rlr_b : rlr_c;
            EpiRowMajor e4{out, (long long)nij * m, 0};
            gemm_begin();
            if (split)
                split_gemm4_op(ctx, sx == 2 ? 1 : 0, rk, 2 * n, (long long)nij * m, e4, &ps.launches);
            else
                gemm_f64(st, sx == 2 ? ctx->d_qbh : ctx->d_qah, 2 * n, 0, rk, (long long)nij * m, 0, 2 * m, nij * m,
                         2 * n, 1, e4), ++ps.launches;
            gemm_end(2.0 * 2 * m * (double)nij * m * 2 * n);
            tr.mark("B: Gaunt GEMM4");
        }
        if (breit) {  // the records need other items' RL: assembled after all chunks
            launch_rl_store(st, split, rlr, rlr_b, rlr_c, m, nij, i0, ps.d_itrmo, -1.0, ctx->d_rl_all);
            ++ps.launches;
            tr.mark("B: Gaunt RL store");
            continue;
        }
        for (int cc = 0; cc < 2 && !breit; ++cc) {
            const int nc = P.ncomp[cc];
            if (nc == 0) continue;
            launch_expand(st, ctx->d_hp, P.P, KK1, i0, nij, ps.d_pidx[cc], nc, nc, m3, false, split, halves);
            ++ps.launches;
            tr.mark("B: expand M_ij(p,q)");
            EpiRK e3{rk, m, (long long)P.comp_off[cc] * nij, rkplane};
            gemm_begin();
            if (split)
                split_gemm3(ctx, cc, m3, nc, nij, e3, &ps.launches);
            else
                gemm_f64(st, m3, 2 * nc, 0, ctx->d_qar[cc], 2 * m, 0, nc * nij, 2 * m, 2 * nc, 1, e3), ++ps.launches;
            gemm_end(2.0 * nc * (double)nij * 2 * m * 2 * nc);
            tr.mark("B: GEMM3");
        }
        if (!breit) {
            EpiRowMajor e4{rlr, (long long)nij * m, 0};
            gemm_begin();
            if (split)
                split_gemm24(ctx, rk, 2 * n, (long long)nij * m, e4, &ps.launches);
            else
                gemm_f64(st, ctx->d_qah, 2 * n, 0, rk, (long long)nij * m, 0, 2 * m, nij * m, 2 * n, 1, e4),
                    ++ps.launches;
            gemm_end(2.0 * 2 * m * (double)nij * m * 2 * n);
            tr.mark("B: slice RK + GEMM4");
        }
        if (halves) {  // rotran's halves: MSUMTIM (ISG = +1) into every item's RL
            launch_rl_store(st, split, rlr, nullptr, nullptr, m, nij, i0, ps.d_itrmo, 1.0, ctx->d_rl_all);
            ++ps.launches;
            tr.mark("B: RL store");
            continue;
        }
        // MDCINT selection for the records of this chunk
        chunk_recs.assign(w.recs.begin() + w.item_rec0[i0], w.recs.begin() + w.item_rec0[i0 + nij]);
        for (int t = i0; t < i0 + nij; ++t)
            for (int r = w.item_rec0[t]; r < w.item_rec0[t + 1]; ++r)
                chunk_recs[r - w.item_rec0[i0]].ijl = t - i0;
        RT_CUDA(cudaMemcpyAsync(d_recs, chunk_recs.data(), chunk_recs.size() * sizeof(EmitRec), cudaMemcpyHostToDevice, st));
        launch_emit(st, split, rlr, m, nij, K, d_recs, (int)chunk_recs.size(), ps.d_kra, ps.d_krb,
                    ps.d_itrmo, ctx->cfg.throut, os);
        ps.launches += 3;
        // the host copy of chunk_recs must outlive the async copy
        RT_CUDA(cudaStreamSynchronize(st));
        tr.mark("B: MDCINT selection");
        stream_out();
    }
    // rotran's halves: the records from the RL of all items (PPSYM)
    for (int i0 = 0; halves && i0 < KK1; i0 += item_chunk) {
        const int nij = std::min(item_chunk, KK1 - i0);
        chunk_recs.assign(w.recs.begin() + w.item_rec0[i0], w.recs.begin() + w.item_rec0[i0 + nij]);
        for (int t = i0; t < i0 + nij; ++t)
            for (int r = w.item_rec0[t]; r < w.item_rec0[t + 1]; ++r)
                chunk_recs[r - w.item_rec0[i0]].ijl = t - i0;
        RT_CUDA(cudaMemcpyAsync(d_recs, chunk_recs.data(), chunk_recs.size() * sizeof(EmitRec), cudaMemcpyHostToDevice, st));
        launch_emit_halves(st, ctx->d_rl_all, m, K, i0, d_recs, (int)chunk_recs.size(), ps.d_item_of, ps.d_kra,
                           ps.d_krb, ctx->cfg.throut, os);
        ps.launches += 3;
        RT_CUDA(cudaStreamSynchronize(st));
        tr.mark("B: records from both halves");
        stream_out();
    }
    if (to_host && ctx->host_defer) {
        ctx->host_inflight = true;  // completed by rt_result_host_wait or the next user of the results
    } else if (to_host) {
        RT_CUDA(cudaStreamSynchronize(ctx->cstream[0]));
        tr.mark("B: last result copies");
    }
    RT_CUDA(cudaGetLastError());
    RT_CUDA(cudaEventRecord(ctx->ev[4], st));
    long long tot[4];
    unsigned long long hstat[8];
    RT_CUDA(cudaMemcpyAsync(tot, d_total, sizeof(tot), cudaMemcpyDeviceToHost, st));
    RT_CUDA(cudaMemcpyAsync(hstat, ps.d_stat, sizeof(hstat), cudaMemcpyDeviceToHost, st));
    RT_CUDA(cudaEventRecord(ctx->ev[5], st));
    RT_CUDA(cudaStreamSynchronize(st));
    if (split) split_check(ctx);
    for (int cc = 0; cc < 4; ++cc) {
        ctx->out_nz[cc] = tot[cc];
        ctx->out_nrec[cc] = w.nrec[cc];
    }
    float ms[5];
    for (int e = 0; e < 5; ++e) RT_CUDA(cudaEventElapsedTime(&ms[e], ctx->ev[e], ctx->ev[e + 1]));
    rt_stats& S = ctx->stats;
    S.ms_upload = ms[0];
    S.ms_scatter = ms[1];
    S.ms_first = ms[2];
    S.ms_second = ms[3];
    S.ms_output = ms[4];
    float tot_ms = 0;
    RT_CUDA(cudaEventElapsedTime(&tot_ms, ctx->ev[0], ctx->ev[5]));
    S.ms_total = tot_ms;
    S.nhalft = (long long)hstat[1];
    for (int cc = 0; cc < 4; ++cc) {
        S.nfinal[cc] = tot[cc];
        S.nrec[cc] = w.nrec[cc];
    }
    S.flops_algorithmic = algorithmic_flops(P, ctx->cfg.breit != 0);
    S.device_bytes = (long long)ctx->dev_peak;
    S.gpu_launches = ps.launches;
    S.gemm_launches = kt.launches;
    S.ms_gemm = kt.total_ms();
    S.flops_gemm_executed = kt.flops;
    S.flops_gemm_algorithmic = kt.alg;
    ctx->transformed = true;
    tr.mark("counts read back");
    tr.print("rt_transform");
    API_CATCH
}

// Ordered spinor pairs related to each Kramers-unique item u = (I,J): the
// half-transformed integral of pair r is t_r(H_u) with
//   (I,J): H_u,  (J,I): conj(H_u),  (Jbar,Ibar): s H_u,  (Ibar,Jbar): s conj(H_u),
// s = sign(ITRMO(I) ITRMO(J)).  relk holds k + m l of each distinct related
// pair (-1: none), relc the factor as +-1 (plain) or +-2 (conjugated).
// Every ordered pair must belong to exactly one item.
static void build_relatives(rt_ctx* c, std::vector<int4>& relk, std::vector<int4>& relc) {
    const Plan& P = c->plan;
    const int m = P.m;
    const size_t KK1 = P.items.size();
    relk.assign(KK1, make_int4(-1, -1, -1, -1));
    relc.assign(KK1, make_int4(0, 0, 0, 0));
    std::vector<int> cover((size_t)m * m, 0);
    for (size_t t = 0; t < KK1; ++t) {
        const int I = P.items[t].I, J = P.items[t].J;
        const int Ib = std::abs(c->itrmo[I]) - 1, Jb = std::abs(c->itrmo[J]) - 1;
        const int s = ((c->itrmo[I] > 0) == (c->itrmo[J] > 0)) ? 1 : -1;
        const int cand[4][3] = {{I, J, 1}, {J, I, 2}, {Jb, Ib, s}, {Ib, Jb, 2 * s}};
        int kk[4] = {-1, -1, -1, -1}, cc[4] = {0, 0, 0, 0}, nk = 0;
        for (auto& r : cand) {
            const int lin = r[0] + m * r[1];
            bool seen = false;
            for (int q = 0; q < nk; ++q) seen = seen || kk[q] == lin;
            if (seen) continue;
            kk[nk] = lin;
            cc[nk] = r[2];
            ++nk;
            ++cover[lin];
        }
        relk[t] = make_int4(kk[0], kk[1], kk[2], kk[3]);
        relc[t] = make_int4(cc[0], cc[1], cc[2], cc[3]);
    }
    for (int v : cover)
        if (v != 1) throw Error(RT_ERR_INTERNAL, "Kramers items do not cover the spinor pairs once");
}

extern "C" int rt_adjoint(rt_ctx* ctx, const double* gamma, double* dedc, double* energy) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    if (!gamma || !dedc) throw Error(RT_ERR_USER, "rt_adjoint: null gamma or dEdC");
    if (ctx->unusable) throw Error(RT_ERR_PROGRAM, UNUSABLE_MSG);
    if (ctx->cfg.breit) throw Error(RT_ERR_USER, "the adjoint is built for the Coulomb transformation");
    if (!ctx->have_coef) throw Error(RT_ERR_USER, "rt_set_coefficients has not been called");
    rq_apply(ctx);
    host_result_wait(ctx);
    Plan& P = ctx->plan;
    cudaStream_t st = ctx->stream;
    const int n = P.n, m = P.m;
    const int KK1 = (int)P.items.size();
    std::vector<int4> relk, relc;
    build_relatives(ctx, relk, relc);
    KTimer& kt = ctx->ktimer;
    kt.reset(st);
    ctx->trace.reset(st);
    ctx->trace.mark("start");
    RT_CUDA(cudaEventRecord(ctx->ev[0], st));
    flush_staged(ctx);
    // the work arena is sized again beside the density
    dfree(ctx, ctx->d_ha);
    ctx->d_ha = nullptr;
    ctx->ha_len = 0;
    ctx->stage.pair_chunk = ctx->stage.item_chunk = 0;
    Pass ps(ctx);
    const size_t ng = (size_t)m * m * m * m;
    double* d_gam = ps.alloc<double>(2 * ng);
    {
        // the density into the internal spinor order
        double* d_tmp = ps.alloc<double>(2 * ng);
        int* d_su = ps.upload(ctx->spin_user.data(), (size_t)m);
        RT_CUDA(cudaMemcpyAsync(d_tmp, gamma, 2 * ng * sizeof(double), cudaMemcpyDefault, st));
        launch_gamma_permute(st, d_tmp, d_su, m, d_gam);
        RT_CUDA(cudaStreamSynchronize(st));
        dfree(ctx, d_tmp);
        ps.tmp.erase(std::find(ps.tmp.begin(), ps.tmp.end(), (void*)d_tmp));
        ps.launches += 1;
    }
    launch_gamma_sym(st, d_gam, m);
    ++ps.launches;
    int4* d_relk = ps.upload(relk.data(), relk.size());
    int4* d_relc = ps.upload(relc.data(), relc.size());
    const long long nacc = (long long)n * 2 * m;
    double* d_acc = ps.alloc<double>((size_t)nacc);
    RT_CUDA(cudaMemsetAsync(d_acc, 0, nacc * sizeof(double), st));
    pass_setup(ps);
    const bool split = ps.split;
    const int s = split ? ctx->cfg.slices : 0;
    auto gemm_begin = [&]() { if (!split) kt.begin(); };
    auto gemm_end = [&](double fl) { if (!split) kt.end(fl, fl); };
    RT_CUDA(cudaEventRecord(ctx->ev[1], st));
    pass_bucketing(ps, false);  // the adjoint differentiates the complete sums
    RT_CUDA(cudaEventRecord(ctx->ev[2], st));
    // recompute the half-transformed integrals, unscreened
    pass_stage_a(ps, 0.0);
    RT_CUDA(cudaEventRecord(ctx->ev[3], st));
    // ---- per item chunk: X_{u,plane} = h_{u,plane} C, then
    //      S += sum_{u,plane} X_{u,plane} Ghat_{u,plane} (split-K over items) ----
    const int G = 8;  // items per partial product of the FP64 path
    const int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
    const double kpc = (double)((ncmax + 31) / 32 * 32);
    // bytes per item of the chunk buffers, and per chunk
    double per_item = 32.0 * n * m + 16.0 * ncmax * ncmax + 64.0 * m * m;
    double fixed = 8.0 * nacc + 8192.0;
    if (split) {
        per_item += 4.0 * m / (double)SPLIT_LONG_BLOCK * 8.0 * nacc;                                  // partials
        per_item += std::max(2.0 * s * n * 4.0 * m, 2.0 * s * 2.0 * ncmax * kpc);    // A slices
        per_item += 2.0 * s * 2.0 * m * 4.0 * m + 8.0 * ncmax;                       // B slices, exps
        per_item += 4.0 * m / (double)SPLIT_LONG_BLOCK * 4.0 * (n + 2.0 * m);                          // split exps
        fixed += 2.0 * s * (n + 2.0 * m) * 64.0 + 8.0 * (n + 2 * m) + 8.0 * nacc + 2048.0;
    } else {
        per_item += 8.0 * nacc / G;
    }
    const double arena = 8.0 * (double)ctx->ha_len;
    int chunk = (int)std::min<double>(KK1, std::floor((arena - fixed) / per_item));
    if (!split && chunk > G) chunk -= chunk % G;
    if (chunk < 1) throw Error(RT_ERR_DIM, "rt_adjoint: work arena too small for one item");
    for (int i0 = 0; i0 < KK1; i0 += chunk) {
        const int nij = std::min(chunk, KK1 - i0);
        const long long Kx = 4LL * m * nij;
        unsigned char* wp = (unsigned char*)ctx->d_ha;
        auto carve = [&](double bytes) {
            unsigned char* r = wp;
            wp += ((size_t)std::ceil(bytes) + 255) & ~(size_t)255;
            return r;
        };
        double* X = (double*)carve(8.0 * Kx * n);
        double* m3 = (double*)carve(16.0 * ncmax * ncmax * nij);
        double* bh = (double*)carve(64.0 * m * m * nij);
        for (int cc = 0; cc < 2; ++cc) {
            const int nc = P.ncomp[cc];
            if (nc == 0) continue;
            launch_expand(st, ctx->d_hp, P.P, KK1, i0, nij, ps.d_pidx[cc], nc, nc, m3);
            ++ps.launches;
            if (split) {
                unsigned char* save = wp;
                __nv_bfloat16* sl = (__nv_bfloat16*)carve(2.0 * s * 2.0 * nc * nij * kpc);
                int* ex = (int*)carve(8.0 * nc * nij);
                split_adj_x(ctx, cc, m3, nc, nij, X, sl, ex, &ps.launches);
                wp = save;
            } else {
                EpiRowMajor ex{X + (size_t)P.comp_off[cc] * nij * 4 * m, 2LL * m, 0};
                gemm_begin();
                gemm_f64(st, m3, nc, 0, ctx->d_qap + (long long)P.comp_off[cc] * 2 * m, 2 * m, 0,
                         2 * nc * nij, 2 * m, nc, 1, ex);
                gemm_end(2.0 * (2.0 * nc * nij) * 2 * m * nc);
                ++ps.launches;
            }
        }
        if (split) {
            const long long Kp = split_adj_kpad(Kx);
            launch_gamma_hat_t(st, d_gam, m, d_relk, d_relc, ps.d_itrmo, i0, nij, Kx, bh);
            ++ps.launches;
            __nv_bfloat16* a_sl = (__nv_bfloat16*)carve(2.0 * s * n * Kp);
            __nv_bfloat16* b_sl = (__nv_bfloat16*)carve(2.0 * s * 2.0 * m * Kp);
            const double nsplit = (double)((Kp + SPLIT_LONG_BLOCK - 1) / SPLIT_LONG_BLOCK);
            int* a_ex = (int*)carve(4.0 * n * nsplit);
            int* b_ex = (int*)carve(8.0 * m * nsplit);
            double* part = (double*)carve(8.0 * nacc * ((Kp / 32 + 31) / 32));
            if ((double)(wp - (unsigned char*)ctx->d_ha) > arena)
                throw Error(RT_ERR_INTERNAL, "rt_adjoint: chunk buffers exceed the work arena");
            const int ks = split_adj_contract(ctx, X, n, Kx, bh, a_sl, a_ex, b_sl, b_ex, part,
                                              &ps.launches);
            launch_partial_sum(st, true, part, ks, nacc, d_acc);
            ++ps.launches;
        } else {
            launch_gamma_hat(st, false, d_gam, m, d_relk, d_relc, ps.d_itrmo, i0, nij, bh);
            ++ps.launches;
            const int nb = nij / G, rem = nij - nb * G;
            double* part = (double*)carve(8.0 * nacc * (nb + 1));
            if ((double)(wp - (unsigned char*)ctx->d_ha) > arena)
                throw Error(RT_ERR_INTERNAL, "rt_adjoint: chunk buffers exceed the work arena");
            const long long K1 = 4LL * m * G;
            gemm_begin();
            if (nb)
                gemm_f64(st, X, Kx, K1, bh, 2 * m, K1 * 2 * m, n, 2 * m, (int)K1, nb,
                         EpiRowMajor{part, 2LL * m, nacc}), ++ps.launches;
            if (rem)
                gemm_f64(st, X + nb * K1, Kx, 0, bh + (size_t)nb * K1 * 2 * m, 2 * m, 0, n, 2 * m,
                         4 * m * rem, 1, EpiRowMajor{part + (size_t)nb * nacc, 2LL * m, 0}), ++ps.launches;
            gemm_end(2.0 * n * 2 * m * (double)Kx);
            launch_partial_sum(st, false, part, nb + (rem > 0 ? 1 : 0), nacc, d_acc);
            ++ps.launches;
        }
    }
    RT_CUDA(cudaGetLastError());
    RT_CUDA(cudaEventRecord(ctx->ev[4], st));
    std::vector<double> acc((size_t)nacc);
    RT_CUDA(cudaMemcpyAsync(acc.data(), d_acc, nacc * sizeof(double), cudaMemcpyDeviceToHost, st));
    RT_CUDA(cudaEventRecord(ctx->ev[5], st));
    RT_CUDA(cudaStreamSynchronize(st));
    if (split) split_check(ctx);
    // dE/dRe C + i dE/dIm C = 4 S (rows back in the caller's AO order);
    // E = sum conj(C) S (E is of degree 2 in conj(C))
    std::vector<double> out((size_t)2 * n * m);
    double e = 0.0;
    for (int p = 0; p < n; ++p) {
        const double* row = acc.data() + (size_t)P.ao_sorted[p] * 2 * m;
        for (int x = 0; x < m; ++x) {
            const double sr = row[x], si = row[m + x];
            const size_t o = 2 * ((size_t)p + (size_t)n * x);
            const size_t ou = 2 * ((size_t)p + (size_t)n * ctx->spin_user[x]);  // caller's column
            out[ou] = 4.0 * sr;
            out[ou + 1] = 4.0 * si;
            e += ctx->qa[o] * sr + ctx->qa[o + 1] * si;
        }
    }
    RT_CUDA(cudaMemcpy(dedc, out.data(), out.size() * sizeof(double), cudaMemcpyDefault));
    if (energy) *energy = e;
    ctx->trace.mark("dE/dC to the caller");
    ctx->trace.print("rt_adjoint");
    float ms[5];
    for (int q = 0; q < 5; ++q) RT_CUDA(cudaEventElapsedTime(&ms[q], ctx->ev[q], ctx->ev[q + 1]));
    rt_stats& S = ctx->stats;
    S.ms_upload = ms[0];
    S.ms_scatter = ms[1];
    S.ms_first = ms[2];
    S.ms_second = ms[3];
    S.ms_output = ms[4];
    float tot_ms = 0;
    RT_CUDA(cudaEventElapsedTime(&tot_ms, ctx->ev[0], ctx->ev[5]));
    S.ms_total = tot_ms;
    double fx = 0.0;
    for (int cc = 0; cc < 2; ++cc) fx += 8.0 * (double)P.ncomp[cc] * P.ncomp[cc] * m;
    S.flops_algorithmic = (algorithmic_flops(P, false) - (double)KK1 * (fx + 8.0 * n * (double)m * m)) +
                          (double)KK1 * (fx + 16.0 * n * (double)m * m);
    S.device_bytes = (long long)ctx->dev_peak;
    S.gpu_launches = ps.launches;
    S.gemm_launches = kt.launches;
    S.ms_gemm = kt.total_ms();
    S.flops_gemm_executed = kt.flops;
    S.flops_gemm_algorithmic = kt.alg;
    API_CATCH
}

// ---------------------------------------------------------------------------
// batched transforms: many contexts, each planned as a single chunk, run
// stage by stage with one persistent grouped launch per GEMM stage, the
// whole sequence captured once as a CUDA graph and replayed
// ---------------------------------------------------------------------------
namespace {

struct BatchInst {
    rt_ctx* c = nullptr;
    std::unique_ptr<Pass> ps;
    unsigned long long gen = 0;
    long long* d_total = nullptr;
    long long* d_off[4] = {nullptr, nullptr, nullptr, nullptr};
    EmitRec* d_recs = nullptr;
    int nrecs = 0;
    std::vector<ExpandJob*> d_jobs;
    std::vector<size_t> jobs_smem;
    float* d_pthr = nullptr;
    std::vector<int> covered;
    OutStreams os{};
};

}  // namespace

struct rt_batch {
    std::vector<BatchInst> inst;
    int device = 0;
    cudaStream_t st = nullptr;
    int* d_err = nullptr;
    std::vector<SplitGroup*> g1, g2;  // per pair-group stage
    SplitGroup* g3[2] = {nullptr, nullptr};
    SplitGroup* g4 = nullptr;
    std::vector<SplitGroup*> all;     // enqueue order
    std::vector<int> bn;              // tile width per group of `all`
    cudaEvent_t ev[2] = {nullptr, nullptr};
    std::vector<cudaEvent_t> gev;     // around each grouped launch (tuning)
    // per-instance kernels of a stage run on side streams forked from st
    static constexpr int NSIDE = 8;
    cudaStream_t side[NSIDE] = {};
    cudaEvent_t fork = nullptr, join[NSIDE] = {};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool tuned = false;
    int launches = 0;
    rt_batch_stats stats{};
    std::string err;
    ~rt_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (SplitGroup* g : all) split_group_free(g);
        for (auto e : ev) if (e) cudaEventDestroy(e);
        for (auto e : gev) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        for (int i = 0; i < NSIDE; ++i) {
            if (join[i]) cudaEventDestroy(join[i]);
            if (side[i]) cudaStreamDestroy(side[i]);
        }
        if (d_err) cudaFree(d_err);
        inst.clear();
        if (st) cudaStreamDestroy(st);
    }
};

namespace {

// All kernels of one batched run on b->st (no host synchronisation, so the
// sequence can be captured); with `timed`, events around each grouped launch.
void batch_enqueue(rt_batch* b, bool timed) {
    cudaStream_t st = b->st;
    int& L = b->launches;
    L = 0;
    size_t gi = 0;
    auto group = [&](SplitGroup* g) {
        if (!g || split_group_size(g) == 0) { ++gi; return; }
        if (timed) RT_CUDA(cudaEventRecord(b->gev[2 * gi], st));
        split_group_launch(g, b->bn[gi], st, b->d_err);
        if (timed) RT_CUDA(cudaEventRecord(b->gev[2 * gi + 1], st));
        ++L;
        ++gi;
    };
    // run fn(instance, stream) for every instance on the side streams
    auto each = [&](auto fn) {
        RT_CUDA(cudaEventRecord(b->fork, st));
        for (int s = 0; s < rt_batch::NSIDE; ++s) RT_CUDA(cudaStreamWaitEvent(b->side[s], b->fork, 0));
        for (size_t i = 0; i < b->inst.size(); ++i) fn(b->inst[i], b->side[i % rt_batch::NSIDE]);
        for (int s = 0; s < rt_batch::NSIDE; ++s) {
            RT_CUDA(cudaEventRecord(b->join[s], b->side[s]));
            RT_CUDA(cudaStreamWaitEvent(st, b->join[s], 0));
        }
    };
    // ---- bucketing ----
    each([&](BatchInst& I, cudaStream_t ss) {
        rt_ctx* c = I.c;
        const Plan& P = c->plan;
        const DeviceTabs& T = I.ps->T;
        RT_CUDA(cudaMemsetAsync(I.d_total, 0, 4 * sizeof(long long), ss));
        RT_CUDA(cudaMemsetAsync(I.ps->d_stat, 0, 8 * sizeof(unsigned long long), ss));
        ScatterTabs tb{P.n, c->cfg.mfil, P.nblk, T.pq_read, T.pair_of_orig, T.pair_group, T.pg_start,
                       T.pg_size, T.ao_block, T.ao_pos, T.blk_size, T.g1_of, T.g1_kblk,
                       T.jb_base, T.jb_band, T.pg_bbase, T.pg_njobs};
        launch_bucket(ss, c->d_rint, c->d_l2, c->d_l1, c->n_int, I.ps->d_roff, I.ps->d_rmeta,
                      (int)c->rec_off.size(), tb, P.P, c->d_bcount, c->d_boff, c->d_bval,
                      c->d_brs, P.nbuckets, c->d_jstart, c->d_jcount, c->d_jval, c->d_jrs,
                      (unsigned int*)I.ps->d_stat);
        L += c->n_int > 0 ? 3 : 1;
    });
    // ---- first half, pair-group stage by stage ----
    for (size_t g = 0; g < b->g1.size(); ++g) {
        each([&](BatchInst& I, cudaStream_t ss) {
            rt_ctx* c = I.c;
            const Plan& P = c->plan;
            if (g >= P.pgroups.size()) return;
            const int n = P.n, m = P.m, npc = P.pgroups[g].size;
            if (I.covered[g] < n)
                RT_CUDA(cudaMemsetAsync(c->d_ha, 0, (size_t)2 * n * m * npc * sizeof(double), ss));
            if (!P.pg_jobs[g].empty()) {
                launch_expand_rows(ss, c->cfg.slices, c->d_jval, c->d_jrs, c->d_jstart, c->d_jcount,
                                   I.d_jobs[g],
                                   P.pg_njobs[g], P.pg_bbase[g], npc, I.jobs_smem[g], nullptr,
                                   split_a1_slices(c), split_a1_exps(c));
                ++L;
            }
        });
        group(b->g1[g]);
        each([&](BatchInst& I, cudaStream_t ss) {
            rt_ctx* c = I.c;
            const Plan& P = c->plan;
            if (g >= P.pgroups.size()) return;
            split_prep_gemm24(c, c->d_ha, 2 * P.n, (long long)P.m * P.pgroups[g].size, ss, &L);
        });
        group(b->g2[g]);
        each([&](BatchInst& I, cudaStream_t ss) {
            rt_ctx* c = I.c;
            const Plan& P = c->plan;
            if (g >= P.pgroups.size()) return;
            const int n = P.n, m = P.m, npc = P.pgroups[g].size;
            const int KK1 = (int)P.items.size();
            double* ri = c->d_ha + (size_t)2 * n * m * I.ps->pair_chunk;
            launch_tr_select(ss, true, ri, m, npc, P.pgroups[g].start, P.P, I.ps->d_items,
                             I.ps->d_isign, KK1, I.ps->d_pvmx, I.d_pthr, c->cfg.thrgen, c->d_hp,
                             I.ps->d_stat + 1);
            L += (KK1 + 65534) / 65535;
        });
    }
    // ---- second half ----
    for (int cc = 0; cc < 2; ++cc) {
        each([&](BatchInst& I, cudaStream_t ss) {
            rt_ctx* c = I.c;
            const Plan& P = c->plan;
            const int nc = P.ncomp[cc], KK1 = (int)P.items.size();
            if (nc == 0) return;
            launch_expand(ss, c->d_hp, P.P, KK1, 0, KK1, I.ps->d_pidx[cc], nc, nc, c->d_ha);
            ++L;
            split_prep_gemm3(c, c->d_ha, nc, KK1, ss, &L);
        });
        group(b->g3[cc]);
    }
    each([&](BatchInst& I, cudaStream_t ss) {
        rt_ctx* c = I.c;
        const Plan& P = c->plan;
        const int n = P.n, m = P.m, KK1 = (int)P.items.size();
        const int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
        double* rk = c->d_ha + (size_t)2 * ncmax * ncmax * I.ps->item_chunk;
        split_prep_gemm24(c, rk, 2 * n, (long long)KK1 * m, ss, &L);
    });
    group(b->g4);
    each([&](BatchInst& I, cudaStream_t ss) {
        rt_ctx* c = I.c;
        const Plan& P = c->plan;
        const int n = P.n, m = P.m, KK1 = (int)P.items.size();
        const int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
        double* rlr = c->d_ha + (size_t)2 * ncmax * ncmax * I.ps->item_chunk +
                      (size_t)2 * n * m * I.ps->item_chunk;
        launch_emit(ss, true, rlr, m, KK1, P.K, I.d_recs, I.nrecs, I.ps->d_kra, I.ps->d_krb,
                    I.ps->d_itrmo, c->cfg.throut, I.os);
        L += 3;
    });
    RT_CUDA(cudaGetLastError());
}

}  // namespace

extern "C" int rt_batch_create(rt_batch** out, rt_ctx* const* ctxs, int count) {
    if (!out) return RT_ERR_USER;
    *out = nullptr;
    std::unique_ptr<rt_batch> b(new (std::nothrow) rt_batch());
    if (!b) return RT_ERR_PROGRAM;
    rt_batch* B = b.get();
    try {
        if (count < 1 || !ctxs) throw Error(RT_ERR_USER, "empty batch");
        RT_CUDA(cudaGetDevice(&B->device));
        RT_CUDA(cudaStreamCreateWithFlags(&B->st, cudaStreamNonBlocking));
        RT_CUDA(cudaMalloc(&B->d_err, sizeof(int)));
        RT_CUDA(cudaMemset(B->d_err, 0, sizeof(int)));
        for (int i = 0; i < 2; ++i) RT_CUDA(cudaEventCreate(&B->ev[i]));
        RT_CUDA(cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming));
        for (int i = 0; i < rt_batch::NSIDE; ++i) {
            RT_CUDA(cudaStreamCreateWithFlags(&B->side[i], cudaStreamNonBlocking));
            RT_CUDA(cudaEventCreateWithFlags(&B->join[i], cudaEventDisableTiming));
        }
        size_t gmax = 0;
        for (int i = 0; i < count; ++i) {
            rt_ctx* c = ctxs[i];
            if (!c) throw Error(RT_ERR_USER, "null context in batch");
            if (c->device != B->device) throw Error(RT_ERR_USER, "batch contexts on different devices");
            rq_apply(c);
            if (!c->have_coef) throw Error(RT_ERR_USER, "rt_set_coefficients has not been called");
            if (c->cfg.breit) throw Error(RT_ERR_USER, "batched transforms are Coulomb only");
            if (c->cfg.half_buckets)
                throw Error(RT_ERR_USER, "batched transforms use complete sums (half_buckets = 0)");
            if (c->cfg.precision != RT_PREC_SPLIT_BF16)
                throw Error(RT_ERR_USER, "batched transforms use precision RT_PREC_SPLIT_BF16");
            for (int j = 0; j < i; ++j)
                if (ctxs[j] == c) throw Error(RT_ERR_USER, "context twice in one batch");
            flush_staged(c);
            gmax = std::max(gmax, c->plan.pgroups.size());
        }
        B->inst.resize(count);
        for (int i = 0; i < count; ++i) {
            BatchInst& I = B->inst[i];
            rt_ctx* c = ctxs[i];
            I.c = c;
            I.gen = c->gen;
            I.ps.reset(new Pass(c));
            pass_setup(*I.ps, true);
            Pass& ps = *I.ps;
            Plan& P = c->plan;
            Work& w = W(c);
            I.d_total = ps.alloc<long long>(4);
            I.d_pthr = pass_pair_thr(ps, c->cfg.thrgen);
            for (int cc = 0; cc < 4; ++cc) I.d_off[cc] = ps.alloc<long long>(std::max(1LL, w.nrec[cc]));
            std::vector<EmitRec> recs(w.recs);
            for (size_t t = 0; t < P.items.size(); ++t)
                for (int r = w.item_rec0[t]; r < w.item_rec0[t + 1]; ++r) recs[r].ijl = (int)t;
            I.nrecs = (int)recs.size();
            I.d_recs = ps.upload(recs.data(), recs.size());
            for (int cc = 0; cc < 4; ++cc) {
                I.os.cnt[cc] = c->d_hdr[cc];
                I.os.off[cc] = I.d_off[cc];
                I.os.idx[cc] = c->d_oidx[cc];
                I.os.val[cc] = c->d_oval[cc];
            }
            I.os.total = I.d_total;
            I.d_jobs.assign(P.pgroups.size(), nullptr);
            I.jobs_smem.assign(P.pgroups.size(), 0);
            I.covered.assign(P.pgroups.size(), 0);
            for (size_t g = 0; g < P.pgroups.size(); ++g) {
                const auto& jv = P.pg_jobs[g];
                I.d_jobs[g] = ps.upload(jv.data(), std::max<size_t>(1, jv.size()));
                for (auto& j : jv) I.jobs_smem[g] = std::max(I.jobs_smem[g], (size_t)(j.r_hi - j.r_lo) * j.nk * 8);
                for (auto& gg : P.g1)
                    if (gg.pg == (int)g) I.covered[g] += P.blk_size[gg.rblk];
            }
        }
        RT_CUDA(cudaDeviceSynchronize());
        // grouped GEMM stages
        B->g1.assign(gmax, nullptr);
        B->g2.assign(gmax, nullptr);
        for (size_t g = 0; g < gmax; ++g) {
            B->g1[g] = split_group_new(0);
            B->all.push_back(B->g1[g]);
            B->g2[g] = split_group_new(1);
            B->all.push_back(B->g2[g]);
            for (BatchInst& I : B->inst) {
                rt_ctx* c = I.c;
                const Plan& P = c->plan;
                if (g >= P.pgroups.size()) continue;
                const int n = P.n, m = P.m, npc = P.pgroups[g].size;
                const long long plane = (long long)n * m * npc;
                for (auto& gg : P.g1)
                    if (gg.pg == (int)g)
                        split_group_add_gemm1(B->g1[g], c, gg, npc, EpiHA{c->d_ha, P.blk_start[gg.rblk], m, npc, plane});
                double* ri = c->d_ha + (size_t)2 * n * m * I.ps->pair_chunk;
                split_group_add_gemm2_kramers(B->g2[g], c, 2 * n, (long long)m * npc,
                                              EpiRowMajor{ri, (long long)m * npc, 0});
            }
        }
        for (int cc = 0; cc < 2; ++cc) {
            B->g3[cc] = split_group_new(2);
            B->all.push_back(B->g3[cc]);
            for (BatchInst& I : B->inst) {
                rt_ctx* c = I.c;
                const Plan& P = c->plan;
                const int n = P.n, m = P.m, nc = P.ncomp[cc], KK1 = (int)P.items.size();
                if (nc == 0) continue;
                const int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
                double* rk = c->d_ha + (size_t)2 * ncmax * ncmax * I.ps->item_chunk;
                split_group_add_gemm3(B->g3[cc], c, cc, nc, KK1,
                                      EpiRK{rk, m, (long long)P.comp_off[cc] * KK1, (long long)n * KK1 * m});
            }
        }
        B->g4 = split_group_new(1);
        B->all.push_back(B->g4);
        for (BatchInst& I : B->inst) {
            rt_ctx* c = I.c;
            const Plan& P = c->plan;
            const int n = P.n, m = P.m, KK1 = (int)P.items.size();
            const int ncmax = std::max(P.ncomp[0], P.ncomp[1]);
            double* rlr = c->d_ha + (size_t)2 * ncmax * ncmax * I.ps->item_chunk +
                          (size_t)2 * n * m * I.ps->item_chunk;
            split_group_add_gemm24(B->g4, c, 2 * n, (long long)KK1 * m, EpiRowMajor{rlr, (long long)KK1 * m, 0});
        }
        for (SplitGroup* g : B->all) split_group_build(g, B->inst[0].c);
        B->bn.assign(B->all.size(), 128);
        B->gev.resize(2 * B->all.size());
        for (auto& e : B->gev) RT_CUDA(cudaEventCreate(&e));
        B->stats.instances = count;
        for (BatchInst& I : B->inst) B->stats.flops_algorithmic += algorithmic_flops(I.c->plan, false);
        for (SplitGroup* g : B->all) B->stats.flops_gemm_executed += split_group_flops(g, true);
    } catch (const Error& e) {
        rt::set_thread_error(e.msg);
        return e.code;
    } catch (const std::exception& e) {
        rt::set_thread_error(e.what());
        return RT_ERR_PROGRAM;
    }
    *out = b.release();
    return RT_OK;
}

namespace {

// Tile-width cache of the batch tuner: a flat JSON object {"shape": width}
// in the file named by RT_TUNE_CACHE (shape from split_group_shape).
std::vector<std::pair<std::string, int>> tune_cache_read(const char* path) {
    std::vector<std::pair<std::string, int>> out;
    FILE* f = std::fopen(path, "rb");
    if (!f) return out;
    std::string t;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0 && t.size() < (1u << 20)) t.append(buf, n);
    std::fclose(f);
    size_t i = 0;
    while ((i = t.find('"', i)) != std::string::npos) {
        const size_t j = t.find('"', i + 1);
        if (j == std::string::npos) break;
        const std::string key = t.substr(i + 1, j - i - 1);
        size_t k = j + 1;
        while (k < t.size() && (t[k] == ' ' || t[k] == ':' || t[k] == '\n' || t[k] == '\t')) ++k;
        const int v = std::atoi(t.c_str() + k);
        if (v == 64 || v == 128) out.push_back({key, v});
        i = j + 1;
    }
    return out;
}

void tune_cache_write(const char* path, const std::vector<std::pair<std::string, int>>& add) {
    std::vector<std::pair<std::string, int>> all = tune_cache_read(path);
    for (const auto& kv : add) {
        bool found = false;
        for (auto& e : all)
            if (e.first == kv.first) { e.second = kv.second; found = true; }
        if (!found) all.push_back(kv);
    }
    const std::string tmp = std::string(path) + ".tmp";
    FILE* f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;  // the cache is an optimisation: an unwritable path only costs the tuning
    std::fprintf(f, "{\n");
    for (size_t i = 0; i < all.size(); ++i)
        std::fprintf(f, "  \"%s\": %d%s\n", all[i].first.c_str(), all[i].second, i + 1 < all.size() ? "," : "");
    std::fprintf(f, "}\n");
    std::fclose(f);
    std::rename(tmp.c_str(), path);
}

}  // namespace

extern "C" int rt_batch_run(rt_batch* b) {
    if (!b) return RT_ERR_USER;
    try {
        for (BatchInst& I : b->inst) {
            if (I.c->unusable) throw Error(RT_ERR_PROGRAM, UNUSABLE_MSG);
            if (I.c->gen != I.gen || I.c->rq.pending)
                throw Error(RT_ERR_MISMATCH, "a context of the batch changed after rt_batch_create");
        }
        for (BatchInst& I : b->inst) {
            host_result_wait(I.c);
            I.c->transformed = false;  // rewritten from here on
        }
        // tile widths from the cache when every stage's shape is in it
        const char* cache = std::getenv("RT_TUNE_CACHE");
        bool cached = false;
        if (!b->tuned && cache && *cache) {
            const auto entries = tune_cache_read(cache);
            cached = true;
            std::vector<int> bn(b->all.size(), 128);
            for (size_t i = 0; i < b->all.size() && cached; ++i) {
                if (split_group_size(b->all[i]) == 0) continue;
                const std::string key = split_group_shape(b->all[i]);
                bool hit = false;
                for (const auto& e : entries)
                    if (e.first == key) { bn[i] = e.second; hit = true; }
                cached = hit;
            }
            if (cached) {
                b->stats.tile128 = b->stats.tile64 = 0;
                for (size_t i = 0; i < b->all.size(); ++i) {
                    b->bn[i] = bn[i];
                    if (split_group_size(b->all[i]) > 0) ++(bn[i] == 64 ? b->stats.tile64 : b->stats.tile128);
                }
                b->stats.ms_tune = 0.0;  // no tuning runs
            }
        }
        if (!b->tuned && !cached) {
            // tile width per grouped stage: time every stage at 128 and at 64
            std::vector<float> ms[2];
            cudaEvent_t a, z;
            RT_CUDA(cudaEventCreate(&a));
            RT_CUDA(cudaEventCreate(&z));
            RT_CUDA(cudaEventRecord(a, b->st));
            for (int v = 0; v < 2; ++v) {
                std::fill(b->bn.begin(), b->bn.end(), v == 0 ? 128 : 64);
                batch_enqueue(b, true);
                RT_CUDA(cudaStreamSynchronize(b->st));
                ms[v].assign(b->all.size(), 0.f);
                for (size_t i = 0; i < b->all.size(); ++i)
                    if (split_group_size(b->all[i]) > 0)
                        RT_CUDA(cudaEventElapsedTime(&ms[v][i], b->gev[2 * i], b->gev[2 * i + 1]));
            }
            RT_CUDA(cudaEventRecord(z, b->st));
            RT_CUDA(cudaEventSynchronize(z));
            float tune_ms = 0.f;
            RT_CUDA(cudaEventElapsedTime(&tune_ms, a, z));
            cudaEventDestroy(a);
            cudaEventDestroy(z);
            b->stats.tile128 = b->stats.tile64 = 0;
            for (size_t i = 0; i < b->all.size(); ++i) {
                if (split_group_size(b->all[i]) == 0) continue;
                b->bn[i] = ms[1][i] < ms[0][i] ? 64 : 128;
                ++(b->bn[i] == 64 ? b->stats.tile64 : b->stats.tile128);
            }
            b->stats.ms_tune = tune_ms;
            if (cache && *cache) {
                std::vector<std::pair<std::string, int>> add;
                for (size_t i = 0; i < b->all.size(); ++i)
                    if (split_group_size(b->all[i]) > 0) add.push_back({split_group_shape(b->all[i]), b->bn[i]});
                tune_cache_write(cache, add);
            }
        }
        if (!b->tuned) {
            // capture the tuned sequence once
            RT_CUDA(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
            try {
                batch_enqueue(b, false);
            } catch (...) {
                cudaGraph_t g = nullptr;
                cudaStreamEndCapture(b->st, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            RT_CUDA(cudaStreamEndCapture(b->st, &b->graph));
            RT_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
            size_t nodes = 0;
            RT_CUDA(cudaGraphGetNodes(b->graph, nullptr, &nodes));
            b->stats.graph_nodes = (int)nodes;
            b->stats.kernel_launches = b->launches;
            b->tuned = true;
        }
        RT_CUDA(cudaEventRecord(b->ev[0], b->st));
        RT_CUDA(cudaGraphLaunch(b->exec, b->st));
        RT_CUDA(cudaEventRecord(b->ev[1], b->st));
        RT_CUDA(cudaStreamSynchronize(b->st));
        float ms = 0.f;
        RT_CUDA(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
        b->stats.ms_last = ms;
        int e = 0;
        RT_CUDA(cudaMemcpy(&e, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) {
            bool unconfirmed = false;
            const std::string msg = split_status_text(e, &unconfirmed);
            if (unconfirmed)
                for (BatchInst& I : b->inst) I.c->unusable = true;
            RT_CUDA(cudaMemset(b->d_err, 0, sizeof(int)));
            throw Error(RT_ERR_PROGRAM, "grouped " + msg);
        }
        int grouped = 0;
        for (SplitGroup* g : b->all) grouped += split_group_size(g) > 0 ? 1 : 0;
        b->stats.grouped_launches = grouped;
        for (BatchInst& I : b->inst) {
            rt_ctx* c = I.c;
            long long tot[4];
            unsigned long long hs[8];
            RT_CUDA(cudaMemcpy(tot, I.d_total, sizeof(tot), cudaMemcpyDeviceToHost));
            RT_CUDA(cudaMemcpy(hs, I.ps->d_stat, sizeof(hs), cudaMemcpyDeviceToHost));
            if (hs[0] & ST_BAD_LABEL)
                throw Error(RT_ERR_USER, "integral label outside 1..NSC or pq label with q > p");
            if (hs[0] & ST_BAD_BLOCK)
                throw Error(RT_ERR_USER, "integral outside the (LL|LL)/(SS|LL)/(SS|SS) or irrep block structure");
            Work& w = W(c);
            for (int cc = 0; cc < 4; ++cc) {
                c->out_nz[cc] = tot[cc];
                c->out_nrec[cc] = w.nrec[cc];
                c->stats.nfinal[cc] = tot[cc];
                c->stats.nrec[cc] = w.nrec[cc];
            }
            c->stats.nhalft = (long long)hs[1];
            c->stats.flops_algorithmic = algorithmic_flops(c->plan, c->cfg.breit != 0);
            c->transformed = true;
        }
    } catch (const Error& e) {
        b->err = e.msg;
        return e.code;
    } catch (const std::exception& e) {
        b->err = e.what();
        return RT_ERR_PROGRAM;
    }
    return RT_OK;
}

extern "C" int rt_batch_get_stats(rt_batch* b, rt_batch_stats* out) {
    if (!b || !out) return RT_ERR_USER;
    *out = b->stats;
    return RT_OK;
}

extern "C" const char* rt_batch_last_error(rt_batch* b) { return b ? b->err.c_str() : ""; }

extern "C" void rt_batch_destroy(rt_batch* b) {
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    delete b;
}

extern "C" int rt_result_sizes(rt_ctx* ctx, long long* nrec, long long* nz) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    if (!ctx->transformed) throw Error(RT_ERR_USER, "no transform result");
    long long a = 0, b = 0;
    for (int c = 0; c < 4; ++c) { a += ctx->out_nrec[c]; b += ctx->out_nz[c]; }
    if (nrec) *nrec = a;
    if (nz) *nz = b;
    API_CATCH
}

namespace {

// One pass of tmoone's Fock build over the context's records: MFDFOCK's
// files 1..MFIL with FOCK's terms, or MFDBREIT's file 4 with GAUNT's.  The
// chunk list (records cut into <= 4096 integrals, one block each) is kept
// while the records are unchanged.
void fock_pass(rt_ctx* ctx, bool gaunt, int nmat, const double* dens, double* fock, bool accumulate,
               double* ms_kernel) {
    if (nmat < 1 || nmat > 2) throw Error(RT_ERR_USER, "Fock build: nmat must be 1 or 2");
    if (!dens || !fock) throw Error(RT_ERR_USER, "Fock build: null density or Fock arrays");
    if (ctx->unusable) throw Error(RT_ERR_PROGRAM, UNUSABLE_MSG);
    cudaStream_t st = ctx->stream;
    rq_apply(ctx);
    flush_staged(ctx);
    const int w = gaunt ? 1 : 0;
    if (ctx->fock_gen[w] != ctx->gen) {
        constexpr long long CHUNK = 4096;
        std::vector<FockRec> chunks;
        auto add = [&](size_t r) {
            for (long long o = 0; o < ctx->rec_nt[r]; o += CHUNK)
                chunks.push_back(FockRec{ctx->rec_off[r] + o, std::min(CHUNK, ctx->rec_nt[r] - o), ctx->rec_it[r], 0});
        };
        if (!gaunt) {
            // MFDFOCK reads files 1..MFIL in order (mfdfock.F:68)
            for (int file = 1; file <= std::min(ctx->cfg.mfil, 3); ++file)
                for (size_t r = 0; r < ctx->rec_file.size(); ++r) {
                    if (ctx->rec_file[r] != file || ctx->rec_nt[r] == 0) continue;
                    if (ctx->rec_it[r] < 1 || ctx->rec_it[r] > 14)
                        throw Error(RT_ERR_USER, "integral type outside 1..14 (fock.F:37)");
                    add(r);
                }
        } else {
            // MFDBREIT reads SRTBREI/SRTBREL (mfdbreit.F:66-138)
            for (size_t r = 0; r < ctx->rec_file.size(); ++r) {
                if (ctx->rec_file[r] != 4 || ctx->rec_nt[r] == 0) continue;
                const int it = ctx->rec_it[r];
                if (it != 2 && it != 10 && it != 11 && it != 13 && it != 14)
                    throw Error(RT_ERR_PROGRAM, "INVALID TYPE IN BREIT: type " + std::to_string(it) +
                                                    " (gaunt.F:25-28)");
                add(r);
            }
        }
        if ((long long)chunks.size() >= (1LL << 31)) throw Error(RT_ERR_DIM, "more than 2^31 record chunks");
        dfree(ctx, ctx->d_fock_chunks[w]);
        ctx->d_fock_chunks[w] = nullptr;
        ctx->fock_gen[w] = ~0ull;
        ctx->d_fock_chunks[w] = dalloc<FockRec>(ctx, std::max<size_t>(1, chunks.size()));
        if (!chunks.empty())
            RT_CUDA(cudaMemcpy(ctx->d_fock_chunks[w], chunks.data(), chunks.size() * sizeof(FockRec),
                               cudaMemcpyHostToDevice));
        ctx->n_fock_chunks[w] = (long long)chunks.size();
        ctx->fock_gen[w] = ctx->gen;
    }
    const long long ntri = (long long)ctx->cfg.nsc * (ctx->cfg.nsc + 1) / 2;
    const size_t mat_bytes = (size_t)nmat * 4 * ntri * sizeof(double);
    std::vector<void*> tmp;
    auto* d_dens = (double*)tmp_alloc(ctx, mat_bytes);
    tmp.push_back(d_dens);
    auto* d_fock = (double*)tmp_alloc(ctx, mat_bytes);
    tmp.push_back(d_fock);
    auto* d_bad = (unsigned long long*)tmp_alloc(ctx, sizeof(unsigned long long));
    tmp.push_back(d_bad);
    RT_CUDA(cudaMemcpyAsync(d_dens, dens, mat_bytes, cudaMemcpyDefault, st));
    if (accumulate) RT_CUDA(cudaMemcpyAsync(d_fock, fock, mat_bytes, cudaMemcpyDefault, st));
    else RT_CUDA(cudaMemsetAsync(d_fock, 0, mat_bytes, st));
    RT_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), st));
    RT_CUDA(cudaEventRecord(ctx->ev[0], st));
    launch_fock_skeleton(st, gaunt, ctx->d_rint, ctx->d_l2, ctx->d_l1, (const FockRec*)ctx->d_fock_chunks[w],
                         (int)ctx->n_fock_chunks[w], ctx->cfg.nsc, nmat, d_dens, d_fock, d_bad);
    RT_CUDA(cudaGetLastError());
    RT_CUDA(cudaEventRecord(ctx->ev[1], st));
    unsigned long long bad = 0;
    RT_CUDA(cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, st));
    RT_CUDA(cudaMemcpyAsync(fock, d_fock, mat_bytes, cudaMemcpyDefault, st));
    RT_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    RT_CUDA(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    if (ms_kernel) *ms_kernel = ms;
    tmp_release(ctx, tmp, true);
    if (bad) throw Error(RT_ERR_USER, "integral label outside 1..NSC");
}

}  // namespace

extern "C" int rt_fock_skeleton(rt_ctx* ctx, int nmat, const double* dens, double* fock, double* ms_kernel) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    fock_pass(ctx, false, nmat, dens, fock, false, ms_kernel);
    API_CATCH
}

extern "C" int rt_fock_gaunt(rt_ctx* ctx, int nmat, const double* dens, double* fock, int accumulate,
                             double* ms_kernel) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    fock_pass(ctx, true, nmat, dens, fock, accumulate != 0, ms_kernel);
    API_CATCH
}

extern "C" int rt_set_result_host_deferred(rt_ctx* ctx, int deferred) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    host_result_wait(ctx);
    ctx->host_defer = deferred != 0;
    API_CATCH
}

extern "C" int rt_result_host_wait(rt_ctx* ctx) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    host_result_wait(ctx);
    API_CATCH
}

extern "C" int rt_set_result_host(rt_ctx* ctx, int* const* idx, double* const* val, const long long* cap) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    host_result_wait(ctx);
    ctx->host_on = false;
    const bool on = idx && val;
    for (int c = 0; on && c < 4; ++c)
        if (!cap || cap[c] < 0 || (cap[c] > 0 && (!idx[c] || !val[c])))
            throw Error(RT_ERR_USER, "rt_set_result_host: each class needs buffers for a capacity >= 0");
    for (int c = 0; c < 4; ++c) {
        ctx->host_idx[c] = on ? idx[c] : nullptr;
        ctx->host_val[c] = on ? val[c] : nullptr;
        ctx->host_cap[c] = on ? cap[c] : 0;
    }
    ctx->host_on = on;
    API_CATCH
}

extern "C" int rt_copy_result(rt_ctx* ctx, int* hdr, int* idx, double* val) {
    if (!ctx) return RT_ERR_USER;
    API_TRY
    host_result_wait(ctx);
    if (!ctx->transformed) throw Error(RT_ERR_USER, "no transform result");
    Work& w = W(ctx);
    // every class stream's copies first, one synchronisation
    std::vector<int> cnt[4];
    long long z0 = 0;
    for (int c = 0; c < 4; ++c) {
        const long long nr = ctx->out_nrec[c], nz = ctx->out_nz[c];
        cnt[c].resize(std::max(1LL, nr));
        if (nr) RT_CUDA(cudaMemcpyAsync(cnt[c].data(), ctx->d_hdr[c], nr * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        if (nz && idx) RT_CUDA(cudaMemcpyAsync(idx + 2 * z0, ctx->d_oidx[c], 2 * nz * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        if (nz && val) RT_CUDA(cudaMemcpyAsync(val + 2 * z0, ctx->d_oval[c], 2 * nz * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        z0 += nz;
    }
    RT_CUDA(cudaStreamSynchronize(ctx->stream));
    long long r0 = 0;
    for (int c = 0; c < 4; ++c) {
        if (hdr) {
            long long k = 0;
            for (const EmitRec& r : w.recs) {
                if (r.cls != c) continue;
                int is = -1, js = (c == 0) ? -1 : 1;   // rotran.F:306-328
                hdr[3 * (r0 + k)] = r.ikr * is;
                hdr[3 * (r0 + k) + 1] = r.jkr * js;
                hdr[3 * (r0 + k) + 2] = cnt[c][k];
                ++k;
            }
        }
        r0 += ctx->out_nrec[c];
    }
    API_CATCH
}

extern "C" int rt_get_stats(rt_ctx* ctx, rt_stats* out) {
    if (!ctx || !out) return RT_ERR_USER;
    *out = ctx->stats;
    return RT_OK;
}

extern "C" const char* rt_last_error(rt_ctx* ctx) {
    if (!ctx) return g_create_err.c_str();
    return ctx->err.c_str();
}

extern "C" void rt_destroy(rt_ctx* ctx) {
    if (!ctx) return;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto s : ctx->pstream)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (auto s : ctx->cstream)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (auto& a : ctx->allocs) cudaFree(a.first);
    ctx->allocs.clear();
    split_release(ctx);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int rt_internal_mfil(rt_ctx* c) { return c->cfg.mfil; }
int rt_internal_breit(rt_ctx* c) { return c->cfg.breit; }
int rt_internal_nkr(rt_ctx* c) { return c->cfg.nkr; }
int rt_internal_nsc(rt_ctx* c) { return c->cfg.nsc; }
int rt_internal_nsc1(rt_ctx* c) { return c->cfg.nsc1; }
void rt_internal_set_thread_error(const char* msg) { rt::set_thread_error(msg); }
const int* rt_internal_imoras(rt_ctx* c) { return c->imoras.data(); }
void rt_internal_set_error(rt_ctx* c, const char* msg) { c->err = msg; }

extern "C" int rt_plan(const rt_config* cfg, rt_plan_info* out) {
    if (!out) return RT_ERR_USER;
    std::memset(out, 0, sizeof(*out));
    rt_ctx tmp;
    rt_ctx* ctx = &tmp;
    API_TRY
    check_config(cfg);
    tmp.cfg = *cfg;
    if (cfg->n_irrep == 4) tmp.ao_irrep.assign(cfg->ao_irrep, cfg->ao_irrep + cfg->nsc);
    plan_ao(&tmp);
    const Plan& P = tmp.plan;
    const int K = P.K;
    const long long KK1 = (long long)K * (K + 1);
    out->npairs = P.P;
    out->nitems = KK1;
    plan_expand(&tmp, 0);
    long long a_pp = 0;
    for (long long v : tmp.plan.pg_a_pp) a_pp = std::max(a_pp, v);
    out->expand_bytes_per_pair = a_pp * 8;
    out->hp_bytes = 2 * KK1 * P.P * 8 * (cfg->breit ? 3 : 1);
    const bool all = cfg->throut < 0.0;
    for (int i = 1; i <= K; ++i)
        for (int j = 1; j <= i; ++j) {
            out->nrec[0]++;
            out->elem_cap[0] += set_size(0, i, j, K, all);
            for (int c = 1; c < 4; ++c) {
                out->nrec[c]++;
                out->elem_cap[c] += set_size(c, i, j, K, all);
            }
        }
    out->flops_algorithmic = algorithmic_flops(P, (double)KK1, cfg->breit != 0);
    return RT_OK;
    }
    catch (const rt::Error& e) {
        g_create_err = e.msg;
        return e.code;
    }
    catch (...) {
        g_create_err = "rt_plan failed";
        return RT_ERR_PROGRAM;
    }
}
