// rt_io.cpp -- host-side file formats and checks of the rotran drop-in:
// the SRTTW/SRTLB integral files read by SORT1/GETTW, the MPI version's
// pq-sorted direct-access files SRTPQIL/SRTPQLN read by GETPQ, the MDCINT file
// written by INITTWOE/PPSYM/EXITTWOE (gfortran sequential unformatted
// records with 4-byte length markers), and the KRAMERS pairing check.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

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

// Read one sequential unformatted record (with gfortran subrecords).
// Returns 1 on success, 0 at end of file, -1 on a malformed record.
int read_record(FILE* f, std::vector<char>& buf) {
    buf.clear();
    for (;;) {
        int32_t head;
        size_t got = fread(&head, 4, 1, f);
        if (got != 1) return buf.empty() ? 0 : -1;
        bool more = head < 0;
        long long len = more ? -(long long)head : head;
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

// INTTYP (inttyp.F:1-79): index-coincidence type 1..14 of (i j | k l) with
// the larger pair first.
int inttyp(int i, int j, int k, int l) {
    if (k > j) {
        if (j > l) return i != k ? 13 : 10;
        if (j != l) return k != l ? 14 : 8;
        return i != k ? 11 : 2;
    }
    if (k != l) {
        if (i != j) return j != k ? 12 : 9;
        return j != k ? 5 : 4;
    }
    if (j != k) return i != j ? 7 : 3;
    return i != j ? 6 : 1;
}

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
    long long streams = 0, records = 0, breit_records = 0;
};

std::string rank_name(const char* dir, const char* base, int r) {
    std::string s = std::string(dir) + "/" + base;  // rank 0: no suffix (mfdtwoe.par.F:332-342)
    if (r > 0) s += "." + std::to_string(r);
    return s;
}

// Read the files of ranks 0..nranks-1 (rotran.par.F:430-506, getpq.F:57-125).
// Records are taken in file order; the chains GETPQ follows (INXT links,
// newest first) are checked to partition the records into one chain per
// pq stream, so every record is read exactly once, as GETPQ reads it.
void srtpq_read(const char* dir, int nranks, int nsc, int nsc1, SrtpqSet& out) {
    if (!dir || nranks < 1 || nranks > 999 || nsc < 1 || nsc > 65535 || nsc1 < 0 || nsc1 > nsc)
        throw SrtpqError{RT_ERR_USER, "rt_srtpq: bad arguments"};
    const long long npair = (long long)nsc * (nsc + 1) / 2;
    std::vector<char> rec;
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
        std::vector<char> buf((size_t)irecl);
        for (long long k = 1; k <= lrecco; ++k) {
            const long long pos = (k - 1) * (long long)irecl;
            const size_t want = (size_t)std::min<long long>(irecl, fsize - pos);
            if (pos + 12 > fsize || fread(buf.data(), 1, want, fi.f) != want)
                throw SrtpqError{RT_ERR_EOF, "READ ERROR ON FILE SRTPQIL.*: " + pil + " record " +
                                                 std::to_string(k)};
            int32_t h[3];
            std::memcpy(h, buf.data(), 12);
            const int32_t pq = h[0], nt = h[1], nxt = h[2];
            if (pq < 1 || pq > npair || nt < 0 || nt > nbuf || 12 + 12 * (size_t)nt > want)
                throw SrtpqError{RT_ERR_USER, "bad record header in " + pil + " record " + std::to_string(k)};
            // a link goes to an earlier record of the same stream, and at most
            // one record links to any record (one chain per stream)
            if (nxt < 0 || nxt >= k || (nxt > 0 && (linked[nxt] || ipql[nxt] != pq)))
                throw SrtpqError{RT_ERR_USER, "broken record chain in " + pil + " at record " +
                                                  std::to_string(k)};
            ipql[k] = pq;
            if (nxt > 0) linked[nxt] = 1;
            else ++out.streams;
            ++out.records;
            // the pq pair of the stream (getpq.F:66-67), p >= q
            int ip = (int)(0.5 + 0.5 * std::sqrt(8.0 * pq - 7.0));
            while ((long long)ip * (ip - 1) / 2 >= pq) --ip;
            while ((long long)(ip + 1) * ip / 2 < pq) ++ip;
            const int iq = (int)(pq - (long long)ip * (ip - 1) / 2);
            // Breit records (an SL pq pair) are not Coulomb input (getpq.F:69-75)
            if (ip >= issta && iq <= ilend && nsc > nsc1) {
                ++out.breit_records;
                continue;
            }
            const bool pq_s = ip > nsc1;  // an LL or SS pair from here on
            const char* vals = buf.data() + 12;
            const char* labs = vals + 8 * (size_t)nt;
            for (int e = 0; e < nt; ++e) {
                double v;
                int32_t lab;
                std::memcpy(&v, vals + 8 * (size_t)e, 8);
                std::memcpy(&lab, labs + 4 * (size_t)e, 4);
                const int a = (lab >> 16) & 0xFFFF, b = lab & 0xFFFF;
                if (a < 1 || b < 1 || a > nsc || b > nsc)
                    throw SrtpqError{RT_ERR_USER, "label outside 1..NSC in " + pil + " record " +
                                                      std::to_string(k)};
                const bool rs_s = a > nsc1;
                if (rs_s != (b > nsc1))
                    throw SrtpqError{RT_ERR_USER, "mixed L/S label pair in a Coulomb stream of " + pil};
                // getpq.F:92-96: the type with the larger pair first
                const int it = (a > ip || (a == ip && b >= iq)) ? inttyp(a, b, ip, iq) : inttyp(ip, iq, a, b);
                const int cls = (pq_s && rs_s) ? 3 : (pq_s || rs_s) ? 2 : 1;
                SrtpqGroup& g = out.g[cls - 1][it - 1];
                g.v.push_back(v);
                g.l2.push_back(lab);
                g.l1.push_back((ip << 16) | iq);
            }
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
        srtpq_read(dir, nranks, nsc, nsc1, s);
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
    }
}

// The MPI rotran's input (GETPQ) into a context: one record per (class, type).
extern "C" int rt_read_srtpq_files(rt_ctx* ctx, const char* dir, int nranks) {
    if (!ctx) return RT_ERR_USER;
    try {
        SrtpqSet s;
        srtpq_read(dir, nranks, rt_internal_nsc(ctx), rt_internal_nsc1(ctx), s);
        for (int c = 0; c < 3; ++c)
            for (int t = 0; t < 14; ++t) {
                SrtpqGroup& g = s.g[c][t];
                if (g.v.empty()) continue;
                const int cls = c + 1, it = t + 1;
                const long long n = (long long)g.v.size();
                const int rc = rt_add_ao_records_bulk(ctx, 1, &cls, &n, &it, g.v.data(), g.l2.data(),
                                                      g.l1.data());
                if (rc) return rc;
                std::vector<double>().swap(g.v);
                std::vector<int>().swap(g.l2);
                std::vector<int>().swap(g.l1);
            }
        return RT_OK;
    } catch (const SrtpqError& e) {
        rt_internal_set_error(ctx, e.msg.c_str());
        return e.code;
    } catch (const std::bad_alloc&) {
        rt_internal_set_error(ctx, "rt_read_srtpq_files: out of host memory");
        return RT_ERR_DIM;
    }
}

// SORT1's file loop (sort1.F:118-205) with GETTW's record reads (gettw.F:15-29).
extern "C" int rt_read_srt_files(rt_ctx* ctx, const char* dir) {
    if (!ctx || !dir) return RT_ERR_USER;
    static const char* tw[3] = {"SRTTWLL", "SRTTWSL", "SRTTWSS"};
    static const char* lb[3] = {"SRTLBLL", "SRTLBSL", "SRTLBSS"};
    const int mfil = rt_internal_mfil(ctx);
    std::vector<char> a, b;
    for (int fi = 0; fi < mfil; ++fi) {
        std::string pa = std::string(dir) + "/" + tw[fi], pb = std::string(dir) + "/" + lb[fi];
        File fa(fopen(pa.c_str(), "rb")), fb(fopen(pb.c_str(), "rb"));
        if (!fa.f || !fb.f) {
            rt_internal_set_error(ctx, ("UNABLE TO OPEN SRT FILE " + (fa.f ? pb : pa)).c_str());
            return RT_ERR_EOF;  // sort1.F:227, Q2JOB(1,...)
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

// INITTWOE header (inittwoe.F:139-141), PPSYM records (ppsym.F:89-91) and
// EXITTWOE terminator (exittwoe.F:149).
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
