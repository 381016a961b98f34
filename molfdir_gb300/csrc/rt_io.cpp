// rt_io.cpp -- host-side file formats and checks of the rotran drop-in:
// the SRTTW/SRTLB integral files read by SORT1/GETTW, the MDCINT file
// written by INITTWOE/PPSYM/EXITTWOE (gfortran sequential unformatted
// records with 4-byte length markers), and the KRAMERS pairing check.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
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

}  // namespace

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
