// rt_io.cpp -- host-side file formats and checks of the rotran drop-in:
// the SRTTW/SRTLB integral files read by SORT1/GETTW, the MPI version's
// pq-sorted direct-access files SRTPQIL/SRTPQLN read by GETPQ, the MDCINT file
// written by INITTWOE/PPSYM/EXITTWOE (gfortran sequential unformatted
// records with 4-byte length markers), and the KRAMERS pairing check.
#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <sys/stat.h>

#include "../../include/rotran_gb300.h"
#include "rt_access.h"

namespace {

struct File {
    FILE* f = nullptr;
    explicit File(FILE* x) : f(x) {}
    ~File() {
        if (f) fclose(f);
    }
};

// Bytes left between the read position of f and the end of its file.
long long file_left(FILE* f) {
    struct stat st;
    const long long pos = ftell(f);
    if (pos < 0 || fstat(fileno(f), &st) != 0) return -1;
    return (long long)st.st_size - pos;
}

// Read one sequential unformatted record (with gfortran subrecords).
// Returns 1 on success, 0 at end of file, -1 on a malformed record (also a
// length marker that claims more bytes than the file has left, which is
// rejected before any buffer is sized from it).
int read_record(FILE* f, std::vector<char>& buf) {
    buf.clear();
    for (;;) {
        int32_t head;
        size_t got = fread(&head, 4, 1, f);
        if (got != 1) return buf.empty() ? 0 : -1;
        bool more = head < 0;
        long long len = more ? -(long long)head : head;
        if (len + 4 > file_left(f)) return -1;
        size_t old = buf.size();
        buf.resize(old + len);
        if (len && fread(buf.data() + old, 1, len, f) != (size_t)len) return -1;
        int32_t tail;
        if (fread(&tail, 4, 1, f) != 1) return -1;
        if (!more) return 1;
    }
}

int write_record(FILE* f, const std::vector<const void*>& parts, const std::vector<size_t>& sizes) {
    long long len = 0;
    for (size_t s : sizes) len += (long long)s;
    if (len > 2147483647LL) return -1;  // MDCINT records are far below 2 GB
    int32_t m = (int32_t)len;
    if (fwrite(&m, 4, 1, f) != 1) return -1;
    for (size_t i = 0; i < parts.size(); ++i)
        if (sizes[i] && fwrite(parts[i], 1, sizes[i], f) != sizes[i]) return -1;
    if (fwrite(&m, 4, 1, f) != 1) return -1;
    return 0;
}

// INTTYP (inttyp.F:1-79), the index-coincidence type 1..14 of (i j | k l)
// with the larger pair first, as a table over the seven comparisons its
// decision tree reads: bit 0 k>j, 1 j>l, 2 i!=k, 3 j!=l, 4 k!=l, 5 i!=j, 6 j!=k.
struct InttypTable {
    unsigned char t[128];
    InttypTable() {
        for (int x = 0; x < 128; ++x) {
            const bool kgj = x & 1, jgl = x & 2, ik = x & 4, jl = x & 8, kl = x & 16, ij = x & 32,
                       jk = x & 64;
            int r;
            if (kgj) r = jgl ? (ik ? 13 : 10) : jl ? (kl ? 14 : 8) : (ik ? 11 : 2);
            else if (kl) r = ij ? (jk ? 12 : 9) : (jk ? 5 : 4);
            else r = jk ? (ij ? 7 : 3) : (ij ? 6 : 1);
            t[x] = (unsigned char)r;
        }
    }
    int operator()(int i, int j, int k, int l) const {
        return t[(k > j) | (j > l) << 1 | (i != k) << 2 | (j != l) << 3 | (k != l) << 4 |
                 (i != j) << 5 | (j != k) << 6];
    }
};
const InttypTable inttyp_table;

// ---------------------------------------------------------------------------
// parallel-format input: SRTPQIL[.r] / SRTPQLN[.r]
// ---------------------------------------------------------------------------

struct SrtpqError {
    int code;
    std::string msg;
};

// Integrals of one (file class, type) group, labels as in SRTTW/SRTLB.
struct SrtpqGroup {
    std::vector<double> v;
    std::vector<int> l2, l1;
};

struct SrtpqSet {
    SrtpqGroup g[3][14];  // [class 1..3][type 1..14]
};

// The entries of one block of records, grouped: group g = 14*(class-1) +
// type-1 occupies [start[g], start[g+1]) of v / l2 / l1 -- the layout of
// rt_add_ao_records_bulk with one record per non-empty group.
struct SrtpqBlock {
    // an array of at least n elements (new T[n]: allocated, not
    // value-initialised; every slot is written before it is read)
    template <class T>
    struct Buf {
        std::unique_ptr<T[]> p;
        size_t cap = 0;
        void grow_to(size_t n) {
            if (n > cap) {
                p.reset(new T[n]);
                cap = n;
            }
        }
        T* data() const { return p.get(); }
    };
    Buf<double> v;
    Buf<int> l2, l1;
    long long start[43] = {};
};

std::string rank_name(const char* dir, const char* base, int r) {
    std::string s = std::string(dir) + "/" + base;  // rank 0: no suffix (mfdtwoe.par.F:332-342)
    if (r > 0) s += "." + std::to_string(r);
    return s;
}

// Header of one record after the chain checks: its pq pair, or skip.
struct SrtpqRec {
    int ip = 0, iq = 0, nt = 0;
    bool skip = true;
};

// Decode the entries of records [r0, r1) of a block, calling
// f(group, value, label2, label1) in file order; group = 14*(class-1)+type-1.
// Returns an error text, or nullptr (no allocation: runs on worker threads).
template <class F>
const char* srtpq_decode(const char* block, int irecl, const SrtpqRec* hd, long long r0, long long r1,
                         int nsc, int nsc1, F&& f) {
    for (long long k = r0; k < r1; ++k) {
        const SrtpqRec& h = hd[k];
        if (h.skip) continue;
        const char* vals = block + k * (long long)irecl + 12;
        const char* labs = vals + 8 * (size_t)h.nt;
        const bool pq_s = h.ip > nsc1;  // an LL or SS pair
        const int32_t l1 = (h.ip << 16) | h.iq;
        for (int e = 0; e < h.nt; ++e) {
            double v;
            int32_t lab;
            std::memcpy(&v, vals + 8 * (size_t)e, 8);
            std::memcpy(&lab, labs + 4 * (size_t)e, 4);
            const int a = (lab >> 16) & 0xFFFF, b = lab & 0xFFFF;
            if (a < 1 || b < 1 || a > nsc || b > nsc) return "label outside 1..NSC";
            const bool rs_s = a > nsc1;
            if (rs_s != (b > nsc1)) return "mixed L/S label pair in a Coulomb stream";
            // getpq.F:92-96: the type with the larger pair first
            const bool first = a > h.ip || (a == h.ip && b >= h.iq);
            const int it = first ? inttyp_table(a, b, h.ip, h.iq) : inttyp_table(h.ip, h.iq, a, b);
            const int cls = (pq_s && rs_s) ? 3 : (pq_s || rs_s) ? 2 : 1;
            f(14 * (cls - 1) + it - 1, v, lab, l1);
        }
    }
    return nullptr;
}

// Run fn(w, r0, r1) on t threads over [0, nb); the calling thread takes the
// last part, and the part of any thread that cannot be started.  fn must not
// throw.
template <class F>
void srtpq_parallel(int t, long long nb, F&& fn) {
    std::vector<std::thread> pool;
    pool.reserve((size_t)t);
    int started = 0;
    try {
        for (; started + 1 < t; ++started)
            pool.emplace_back([&, w = started] { fn(w, nb * w / t, nb * (w + 1) / t); });
    } catch (...) {
    }
    for (int w = started; w < t; ++w) fn(w, nb * w / t, nb * (w + 1) / t);
    for (auto& th : pool) th.join();
}

// Read the files of ranks 0..nranks-1 (rotran.par.F:430-506, getpq.F:57-125).
// Records are taken in file order, in blocks: the headers and the chains
// GETPQ follows (INXT links, newest first) are checked sequentially -- the
// links must partition the records into one chain per pq stream, so every
// record is read exactly once, as GETPQ reads it -- then the entries of a
// block are decoded by several threads, each over a contiguous record range,
// and appended in file order.
template <class Sink>
void srtpq_read(const char* dir, int nranks, int nsc, int nsc1, Sink&& sink) {
    if (!dir || nranks < 1 || nranks > 999 || nsc < 1 || nsc > 65535 || nsc1 < 0 || nsc1 > nsc)
        throw SrtpqError{RT_ERR_USER, "rt_srtpq: bad arguments"};
    const long long npair = (long long)nsc * (nsc + 1) / 2;
    const int nthr = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<char> rec;
    SrtpqBlock out;
    SrtpqBlock::Buf<char> block;  // file bytes of a block of records
    for (int r = 0; r < nranks; ++r) {
        const std::string pln = rank_name(dir, "SRTPQLN", r), pil = rank_name(dir, "SRTPQIL", r);
        File fl(fopen(pln.c_str(), "rb")), fi(fopen(pil.c_str(), "rb"));
        if (!fl.f || !fi.f)  // rotran.par.F:443-450
            throw SrtpqError{RT_ERR_EOF, "DIRECT ACCESS OR INFO FILE MISSING: " + (fl.f ? pil : pln)};
        if (read_record(fl.f, rec) != 1 || rec.size() < 24)
            throw SrtpqError{RT_ERR_EOF, "truncated parameter record in " + pln};
        int32_t prm[6];
        std::memcpy(prm, rec.data(), 24);
        const long long lrecco = prm[0];
        const int irecl = prm[1], ilend = prm[3], issta = prm[4], isend = prm[5];
        if (lrecco < 0 || irecl < 24 || (irecl - 12) % 12 != 0)
            throw SrtpqError{RT_ERR_USER, "bad record count or length in " + pln +
                                              " (32-bit layout: IRECL = 12 + 12*NBUFSZ)"};
        if (ilend != nsc1 || (nsc > nsc1 && (issta != nsc1 + 1 || isend != nsc)))
            throw SrtpqError{RT_ERR_USER, "large/small ranges of " + pln + " do not match NSC1/NSC"};
        const int nbuf = (irecl - 12) / 12;
        if (fseek(fi.f, 0, SEEK_END) != 0) throw SrtpqError{RT_ERR_EOF, "cannot size " + pil};
        const long long fsize = ftell(fi.f);
        if (fseek(fi.f, 0, SEEK_SET) != 0) throw SrtpqError{RT_ERR_EOF, "cannot rewind " + pil};
        std::vector<int32_t> ipql(lrecco + 1, 0);
        std::vector<char> linked(lrecco + 1, 0);
        const long long per_block = std::max(1LL, (64LL << 20) / irecl);
        std::vector<SrtpqRec> hd;
        for (long long k0 = 1; k0 <= lrecco; k0 += per_block) {
            const long long nb = std::min(per_block, lrecco - k0 + 1);
            const long long pos = (k0 - 1) * (long long)irecl;
            // the last record may end short of IRECL
            const long long want = std::min<long long>(nb * (long long)irecl, fsize - pos);
            block.grow_to((size_t)nb * irecl);
            if (want < (nb - 1) * (long long)irecl + 12 ||
                fread(block.data(), 1, (size_t)want, fi.f) != (size_t)want)
                throw SrtpqError{RT_ERR_EOF, "READ ERROR ON FILE SRTPQIL.*: " + pil + " records " +
                                                 std::to_string(k0) + ".." + std::to_string(k0 + nb - 1)};
            hd.assign((size_t)nb, SrtpqRec{});
            for (long long i = 0; i < nb; ++i) {
                const long long k = k0 + i;
                int32_t h[3];
                std::memcpy(h, block.data() + i * irecl, 12);
                const int32_t pq = h[0], nt = h[1], nxt = h[2];
                if (pq < 1 || pq > npair || nt < 0 || nt > nbuf ||
                    i * (long long)irecl + 12 + 12LL * nt > want)
                    throw SrtpqError{RT_ERR_USER, "bad record header in " + pil + " record " + std::to_string(k)};
                // a link goes to an earlier record of the same stream, and at
                // most one record links to any record (one chain per stream)
                if (nxt < 0 || nxt >= k || (nxt > 0 && (linked[nxt] || ipql[nxt] != pq)))
                    throw SrtpqError{RT_ERR_USER, "broken record chain in " + pil + " at record " +
                                                      std::to_string(k)};
                ipql[k] = pq;
                if (nxt > 0) linked[nxt] = 1;
                // the pq pair of the stream (getpq.F:66-67), p >= q
                int ip = (int)(0.5 + 0.5 * std::sqrt(8.0 * pq - 7.0));
                while ((long long)ip * (ip - 1) / 2 >= pq) --ip;
                while ((long long)(ip + 1) * ip / 2 < pq) ++ip;
                const int iq = (int)(pq - (long long)ip * (ip - 1) / 2);
                SrtpqRec& x = hd[(size_t)i];
                x.ip = ip;
                x.iq = iq;
                x.nt = nt;
                // Breit records (an SL pq pair) are not Coulomb input (getpq.F:69-75)
                x.skip = ip >= issta && iq <= ilend && nsc > nsc1;
            }
            // count per thread and group, grow the groups once, then write
            // each thread's entries at its offsets (file order is kept)
            const int t = (int)std::min<long long>(nthr, std::max(1LL, nb / 64));
            std::vector<std::array<long long, 42>> cnt((size_t)t), off((size_t)t);
            std::vector<const char*> errs((size_t)t, nullptr);
            srtpq_parallel(t, nb, [&](int w, long long a, long long b) {
                cnt[w].fill(0);
                errs[w] = srtpq_decode(block.data(), irecl, hd.data(), a, b, nsc, nsc1,
                                       [&](int g, double, int32_t, int32_t) { ++cnt[w][g]; });
            });
            for (int w = 0; w < t; ++w)
                if (errs[w]) throw SrtpqError{RT_ERR_USER, std::string(errs[w]) + " in " + pil};
            long long base = 0;
            for (int g = 0; g < 42; ++g) {
                out.start[g] = base;
                for (int w = 0; w < t; ++w) {
                    off[w][g] = base;
                    base += cnt[w][g];
                }
            }
            out.start[42] = base;
            out.v.grow_to((size_t)base);  // reused from block to block
            out.l2.grow_to((size_t)base);
            out.l1.grow_to((size_t)base);
            srtpq_parallel(t, nb, [&](int w, long long a, long long b) {
                std::array<long long, 42> o = off[w];
                srtpq_decode(block.data(), irecl, hd.data(), a, b, nsc, nsc1,
                             [&](int g, double v, int32_t l2, int32_t l1) {
                                 const long long x = o[g]++;
                                 out.v.data()[x] = v;
                                 out.l2.data()[x] = l2;
                                 out.l1.data()[x] = l1;
                             });
            });
            if (base > 0) sink(out);
        }
    }
}

}  // namespace

// Context-free parse of the parallel-format files (see the header).
extern "C" int rt_srtpq_scan(const char* dir, int nranks, int nsc, int nsc1, long long cap,
                             long long* nrec, long long* nint, int* file_class, int* itype,
                             long long* nt, double* rint, int* label2, int* label1) {
    try {
        if (!nrec || !nint) throw SrtpqError{RT_ERR_USER, "rt_srtpq_scan: null count pointers"};
        SrtpqSet s;
        srtpq_read(dir, nranks, nsc, nsc1, [&](const SrtpqBlock& b) {
            for (int g = 0; g < 42; ++g) {
                SrtpqGroup& G = s.g[g / 14][g % 14];
                const long long a = b.start[g], e = b.start[g + 1];
                G.v.insert(G.v.end(), b.v.data() + a, b.v.data() + e);
                G.l2.insert(G.l2.end(), b.l2.data() + a, b.l2.data() + e);
                G.l1.insert(G.l1.end(), b.l1.data() + a, b.l1.data() + e);
            }
        });
        long long nr = 0, ni = 0;
        for (auto& c : s.g)
            for (auto& g : c)
                if (!g.v.empty()) ++nr, ni += (long long)g.v.size();
        *nrec = nr;
        *nint = ni;
        if (ni > cap) return RT_ERR_DIM;  // sizes only
        if (nr && (!file_class || !itype || !nt || !rint || !label2 || !label1))
            throw SrtpqError{RT_ERR_USER, "rt_srtpq_scan: null output arrays"};
        long long k = 0, o = 0;
        for (int c = 0; c < 3; ++c)
            for (int t = 0; t < 14; ++t) {
                const SrtpqGroup& g = s.g[c][t];
                if (g.v.empty()) continue;
                file_class[k] = c + 1;
                itype[k] = t + 1;
                nt[k] = (long long)g.v.size();
                std::memcpy(rint + o, g.v.data(), g.v.size() * 8);
                std::memcpy(label2 + o, g.l2.data(), g.l2.size() * 4);
                std::memcpy(label1 + o, g.l1.data(), g.l1.size() * 4);
                o += nt[k];
                ++k;
            }
        return RT_OK;
    } catch (const SrtpqError& e) {
        rt_internal_set_thread_error(e.msg.c_str());
        return e.code;
    } catch (const std::bad_alloc&) {
        rt_internal_set_thread_error("rt_srtpq_scan: out of host memory");
        return RT_ERR_DIM;
    } catch (...) {
        rt_internal_set_thread_error("rt_srtpq_scan failed");
        return RT_ERR_PROGRAM;
    }
}

// The MPI rotran's input (GETPQ) into a context, streamed: each block of
// records goes to the device as one record per (class, type) it holds.
extern "C" int rt_read_srtpq_files(rt_ctx* ctx, const char* dir, int nranks) {
    if (!ctx) return RT_ERR_USER;
    try {
        int rc = RT_OK;
        srtpq_read(dir, nranks, rt_internal_nsc(ctx), rt_internal_nsc1(ctx), [&](const SrtpqBlock& b) {
            if (rc) return;
            int cls[42], it[42];
            long long nt[42];
            long long nr = 0;
            for (int g = 0; g < 42; ++g)
                if (b.start[g + 1] > b.start[g]) {
                    cls[nr] = g / 14 + 1;
                    it[nr] = g % 14 + 1;
                    nt[nr] = b.start[g + 1] - b.start[g];
                    ++nr;
                }
            rc = rt_add_ao_records_bulk(ctx, nr, cls, nt, it, b.v.data(), b.l2.data(), b.l1.data());
        });
        return rc;
    } catch (const SrtpqError& e) {
        rt_internal_set_error(ctx, e.msg.c_str());
        return e.code;
    } catch (const std::bad_alloc&) {
        rt_internal_set_error(ctx, "rt_read_srtpq_files: out of host memory");
        return RT_ERR_DIM;
    } catch (...) {
        rt_internal_set_error(ctx, "rt_read_srtpq_files failed");
        return RT_ERR_PROGRAM;
    }
}

// SORT1's file loop (sort1.F:60-147) with GETTW's record reads (gettw.F:15-29).
extern "C" int rt_read_srt_files(rt_ctx* ctx, const char* dir) {
    if (!ctx || !dir) return RT_ERR_USER;
    // files 1..MFIL, or the Gaunt file 4 alone (mfdata3.F:15-22, 41-42; sort1.F:55-57)
    static const char* tw[4] = {"SRTTWLL", "SRTTWSL", "SRTTWSS", "SRTBREI"};
    static const char* lb[4] = {"SRTLBLL", "SRTLBSL", "SRTLBSS", "SRTBREL"};
    const bool breit = rt_internal_breit(ctx) != 0;
    const int mfil = rt_internal_mfil(ctx);
    std::vector<char> a, b;
    for (int fi = breit ? 3 : 0; fi < (breit ? 4 : mfil); ++fi) {
        std::string pa = std::string(dir) + "/" + tw[fi], pb = std::string(dir) + "/" + lb[fi];
        File fa(fopen(pa.c_str(), "rb")), fb(fopen(pb.c_str(), "rb"));
        if (!fa.f || !fb.f) {
            rt_internal_set_error(ctx, ("UNABLE TO OPEN SRT FILE " + (fa.f ? pb : pa)).c_str());
            return RT_ERR_EOF;  // sort1.F:169, Q2JOB(1,...)
        }
        for (;;) {
            int ra = read_record(fa.f, a), rb = read_record(fb.f, b);
            if (ra == 0 && rb == 0) {
                rt_internal_set_error(ctx, ("no FINISH record in " + pa).c_str());
                return RT_ERR_EOF;
            }
            if (ra != 1 || rb != 1 || a.size() < 12 || b.size() < 12) {
                rt_internal_set_error(ctx, ("truncated record in " + pa + " / " + pb).c_str());
                return RT_ERR_EOF;
            }
            int32_t nt, it, fin, nt2, it2, fin2;
            std::memcpy(&nt, a.data(), 4);
            std::memcpy(&it, a.data() + 4, 4);
            std::memcpy(&fin, a.data() + 8, 4);
            std::memcpy(&nt2, b.data(), 4);
            std::memcpy(&it2, b.data() + 4, 4);
            std::memcpy(&fin2, b.data() + 8, 4);
            if (nt < 0 || a.size() != 12 + 8 * (size_t)nt || b.size() != 12 + 8 * (size_t)nt2 ||
                nt != nt2 || it != it2) {
                rt_internal_set_error(ctx, ("inconsistent SRTTW/SRTLB records in " + pa).c_str());
                return RT_ERR_USER;
            }
            if (nt > 12288) {  // gettw.F:16 'NT TOO BIG ON SRTTW'
                rt_internal_set_error(ctx, "NT TOO BIG ON SRTTW");
                return RT_ERR_DIM;
            }
            std::vector<double> v(nt);
            std::vector<int> l2(nt), l1(nt);
            if (nt) {
                std::memcpy(v.data(), a.data() + 12, 8 * (size_t)nt);
                std::memcpy(l2.data(), b.data() + 12, 4 * (size_t)nt);
                std::memcpy(l1.data(), b.data() + 12 + 4 * (size_t)nt, 4 * (size_t)nt);
            }
            int rc = rt_add_ao_records(ctx, fi + 1, nt, it, v.data(), l2.data(), l1.data());
            if (rc) return rc;
            if (fin) break;  // GETTW returns FINISH (gettw.F:56)
        }
    }
    return RT_OK;
}

// INITTWOE header (inittwoe.F:21-23), PPSYM records (ppsym.F:89-91) and
// EXITTWOE terminator (exittwoe.F:6).
extern "C" int rt_write_mdcint(rt_ctx* ctx, const char* path, const char* datex10,
                               const char* timex8) {
    if (!ctx || !path) return RT_ERR_USER;
    long long nrec = 0, nz = 0;
    int rc = rt_result_sizes(ctx, &nrec, &nz);
    if (rc) return rc;
    std::vector<int> hdr(3 * (size_t)nrec), idx(2 * (size_t)nz);
    std::vector<double> val(2 * (size_t)nz);
    rc = rt_copy_result(ctx, hdr.data(), idx.data(), val.data());
    if (rc) return rc;
    File f(fopen(path, "wb"));
    if (!f.f) {
        rt_internal_set_error(ctx, (std::string("cannot open ") + path).c_str());
        return RT_ERR_EOF;
    }
    char dt[10], tm[8];
    std::memset(dt, ' ', 10);
    std::memset(tm, ' ', 8);
    if (datex10) std::memcpy(dt, datex10, strnlen(datex10, 10));
    if (timex8) std::memcpy(tm, timex8, strnlen(timex8, 8));
    const int nkr = rt_internal_nkr(ctx);
    const int* im = rt_internal_imoras(ctx);
    if (write_record(f.f, {dt, tm, &nkr, im}, {10, 8, 4, (size_t)8 * nkr})) goto fail;
    {
        long long z = 0;
        std::vector<double> vbuf;
        for (long long r = 0; r < nrec; ++r) {
            const int n = hdr[3 * r + 2];
            if (write_record(f.f, {&hdr[3 * r], &idx[2 * z], &val[2 * z]},
                             {12, (size_t)8 * n, (size_t)16 * n}))
                goto fail;
            z += n;
        }
        int zero[3] = {0, 0, 0};
        if (write_record(f.f, {zero}, {12})) goto fail;
    }
    return RT_OK;
fail:
    rt_internal_set_error(ctx, (std::string("write error on ") + path).c_str());
    return RT_ERR_PROGRAM;
}

// KRAMERS (kramers.F:26-131): find the time-reversal partner of every
// spinor; T QA(i) = QB*(j), T QB(i) = -QA*(j) within PRECIS = 1e-10.
extern "C" int rt_kramers_check(int nsc, int nsp, const double* qa_, const double* qb_, int ld,
                                int* itrmo, double* difmax_out) {
    if (nsc < 1 || nsp < 1 || ld < nsc || !qa_ || !qb_ || !itrmo) return RT_ERR_USER;
    typedef std::complex<double> cd;
    const cd* qa = reinterpret_cast<const cd*>(qa_);
    const cd* qb = reinterpret_cast<const cd*>(qb_);
    auto QA = [&](int i, int m) { return qa[(size_t)i + (size_t)m * ld]; };
    auto QB = [&](int i, int m) { return qb[(size_t)i + (size_t)m * ld]; };
    const double PRECIS = 1e-10;
    double difmax = 0.0;
    for (int i = 0; i < nsp; ++i) itrmo[i] = 0;
    int rc = RT_OK;
    for (int imo = 0; imo < nsp; ++imo) {
        if (itrmo[imo] != 0) continue;
        double rmomax = 0.0, rmoa = 0.0, rmob = 0.0;
        int momax = 0;
        for (int i = 0; i < nsc; ++i) {
            double rmo = std::norm(QA(i, imo)) + std::norm(QB(i, imo));
            if (std::sqrt(rmo) > rmomax) {
                momax = i;
                rmomax = std::sqrt(rmo);
                rmoa = std::abs(QA(i, imo));
                rmob = std::abs(QB(i, imo));
            }
        }
        for (int jmo = 0; jmo < nsp; ++jmo) {
            if (itrmo[jmo] != 0 || rmomax == 0.0) continue;
            double smoa = std::abs(QA(momax, jmo)), smob = std::abs(QB(momax, jmo));
            double dif = (std::fabs(rmoa - smob) + std::fabs(rmob - smoa)) / rmomax;
            if (dif > PRECIS) continue;
            cd phase = rmoa > rmob ? std::conj(QA(momax, imo)) / QB(momax, jmo)
                                   : -std::conj(QB(momax, imo)) / QA(momax, jmo);
            bool ok = true;
            for (int i = 0; i < nsc && ok; ++i) {
                // deviations are recorded once they pass (kramers.F:86-113)
                double d1 = std::abs(std::conj(QA(i, imo)) - QB(i, jmo) * phase);
                if (d1 > PRECIS) { ok = false; break; }
                difmax = std::max(difmax, d1);
                double d2 = std::abs(std::conj(QB(i, imo)) + QA(i, jmo) * phase);
                if (d2 > PRECIS) { ok = false; break; }
                difmax = std::max(difmax, d2);
            }
            if (!ok) continue;
            itrmo[imo] = jmo + 1;
            itrmo[jmo] = -(imo + 1);
            if (std::abs(phase - cd(1.0, 0.0)) > PRECIS) rc = RT_ERR_PROGRAM;  // kramers.F:121-127
            break;
        }
    }
    for (int j = 0; j < nsp; ++j)
        if (itrmo[j] == 0) rc = RT_ERR_PROGRAM;  // kramers.F:133-155
    if (difmax_out) *difmax_out = difmax;
    return rc;
}
