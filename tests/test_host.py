"""Host-side logic of the library: exports, planning, checks, file formats
(no GPU needed; no compute call is made)."""

import os
import re
import struct

import numpy as np
import pytest

from molfdir_gb300 import fortio, rotran, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "rotran_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rt_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    lib = rotran.load()
    names = header_functions()
    assert "rt_transform" in names and "rt_plan" in names
    for name in names:
        assert hasattr(lib, name), name


def test_plan_sizes():
    cfg, _ = rotran.make_config(64, 24, 32)
    pi = rotran.plan(cfg)
    assert pi.npairs == 24 * 25 // 2 + 40 * 41 // 2
    assert pi.nitems == 32 * 33
    assert list(pi.nrec) == [528] * 4
    assert pi.expand_bytes_per_pair == 8 * (24 * 24 + 40 * 40)
    # dense-block FLOPs of both half-transformations
    n, m, k, P = 64, 64, 32, pi.npairs
    f1 = 2 * 2 * m * (P * (24 ** 2 + 40 ** 2)) + P * 8 * n * m * m
    f2 = k * (k + 1) * (8 * (24 ** 2 + 40 ** 2) * m + 8 * n * m * m)
    assert pi.flops_algorithmic == pytest.approx(f1 + f2)


def test_plan_matches_oracle_counts():
    import pyoracle
    p = synth.make_problem(6, 8, 4, seed=2)
    cfg, _ = rotran.make_config(p.n, p.nsc1, p.nkr)
    pi = rotran.plan(cfg)
    img = pyoracle.run(p, throut=-1.0)
    per_class = [int(img.hdr[i * 10:(i + 1) * 10, 2].sum()) for i in range(4)]
    assert per_class == [p.nkr ** 2 * 10] * 4
    img = pyoracle.run(p)
    nz = [int(img.hdr[i * 10:(i + 1) * 10, 2].sum()) for i in range(4)]
    assert all(a <= b for a, b in zip(nz, pi.elem_cap))
    assert nz[0] == pi.elem_cap[0]


@pytest.mark.parametrize("kw,code", [
    (dict(nsc=10, nsc1=10, nkr=3, mfil=3, breit=1), 2),
    (dict(nsc=10, nsc1=0, nkr=3, mfil=3, breit=1), 2),
    (dict(nsc=10, nsc1=4, nkr=3, mfil=3, breit=2), 2),
    (dict(nsc=10, nsc1=4, nkr=3, mfil=1), 2),
    (dict(nsc=70000, nsc1=4, nkr=3, mfil=3), 3),
    (dict(nsc=10, nsc1=11, nkr=3, mfil=3), 2),
    (dict(nsc=10, nsc1=4, nkr=11, mfil=3), 2),
    (dict(nsc=10, nsc1=4, nkr=3, mfil=4), 2),
])
def test_plan_rejects_bad_config(kw, code):
    breit = kw.pop("breit", 0)
    cfg, _ = rotran.make_config(kw["nsc"], kw["nsc1"], kw["nkr"], mfil=kw["mfil"])
    cfg.breit = breit
    with pytest.raises(rotran.RotranError) as e:
        rotran.plan(cfg)
    assert e.value.code == code


def test_plan_reaches_the_reference_basis_limit():
    """N22 = 3000 scalar functions (vecs.inc:4) plan, with 12-bit positions in
    the bucket entries; more than 4095 functions of one component do not."""
    cfg, _ = rotran.make_config(3000, 1500, 8)
    pi = rotran.plan(cfg)
    assert pi.npairs == 2 * (1500 * 1501 // 2)
    cfg, _ = rotran.make_config(5000, 4096, 8)
    with pytest.raises(rotran.RotranError) as e:
        rotran.plan(cfg)
    assert e.value.code == 3


def test_plan_of_the_gaunt_transform():
    """BREIT: the SL pair blocks only (makind.F:91-95), MFIL not used, three
    streams in TRANS2 and the second TRANS1 ZGEMM with QB in the FLOP count."""
    cfg, _ = rotran.make_config(64, 24, 32, mfil=0, breit=True)
    pi = rotran.plan(cfg)
    assert pi.npairs == 24 * 40
    assert pi.nitems == 32 * 33
    n, m, k, P = 64, 64, 32, pi.npairs
    f1 = 2 * 2 * m * (P * 2 * 24 * 40) + 2 * P * 8 * n * m * m
    f2 = k * (k + 1) * 3 * (2 * 8 * 24 * 40 * m + 8 * n * m * m)
    assert pi.flops_algorithmic == pytest.approx(f1 + f2)


def test_create_without_gpu_fails_loudly():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    cfg, _ = rotran.make_config(14, 6, 4)
    with pytest.raises(rotran.RotranError) as e:
        rotran.Rotran(cfg)
    assert e.value.code == 6


def test_kramers_check():
    p = synth.make_problem(5, 7, 4, seed=5)
    itrmo, dif = rotran.kramers_check(p.qa, p.qb)
    assert np.array_equal(itrmo, p.itrmo) and dif < 1e-12
    # a phase on one partner: KRAMERS stops (kramers.F:121-127)
    qa, qb = p.qa.copy(), p.qb.copy()
    qa[:, 1] *= 1j
    qb[:, 1] *= 1j
    with pytest.raises(rotran.RotranError):
        rotran.kramers_check(qa, qb)
    # a spinor without partner (kramers.F:133-155)
    qa, qb = p.qa.copy(), p.qb.copy()
    qa[:, 3] += 1e-3
    with pytest.raises(rotran.RotranError):
        rotran.kramers_check(qa, qb)


def test_srt_files_roundtrip(tmp_path):
    p = synth.make_problem(4, 5, 2, seed=6)
    fortio.write_srt_files(p, str(tmp_path))
    keys = {1: "LL", 2: "SL", 3: "SS"}
    for cls in (1, 2, 3):
        tw, lb = fortio.SRT_NAMES[cls]
        with open(tmp_path / tw, "rb") as fa, open(tmp_path / lb, "rb") as fb:
            for r in p.files[keys[cls]]:
                a, b = fortio.read_record(fa), fortio.read_record(fb)
                nt, it, fin = struct.unpack_from("<iii", a)
                assert (nt, it, bool(fin)) == (r.rint.size, r.it, r.finish)
                assert np.array_equal(np.frombuffer(a, "<f8", nt, 12), r.rint)
                assert np.array_equal(np.frombuffer(b, "<i4", nt, 12), r.label2)
                assert np.array_equal(np.frombuffer(b, "<i4", nt, 12 + 4 * nt), r.label1)
            assert fortio.read_record(fa) is None


def test_record_framing_subrecords(tmp_path):
    path = tmp_path / "x"
    with open(path, "wb") as f:
        # a record split in two gfortran sub-records (negative first marker)
        f.write(struct.pack("<i", -4) + b"abcd" + struct.pack("<i", -4))
        f.write(struct.pack("<i", 3) + b"efg" + struct.pack("<i", 3))
    with open(path, "rb") as f:
        assert fortio.read_record(f) == b"abcdefg"
        assert fortio.read_record(f) is None


def test_header_is_plain_c_and_links(tmp_path):
    """A C caller (the Fortran binding goes through the same ABI) compiles
    against include/rotran_gb300.h as strict C99 and links the library; the
    argument checks that need no device answer without one."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = rotran.load()
    libdir = os.path.dirname(lib._name)
    src = tmp_path / "caller.c"
    src.write_text(
        '#include <stdio.h>\n#include "rotran_gb300.h"\n'
        "int main(void) {\n"
        "  rt_ctx* ctx = 0;\n"
        "  if (rt_transform(0) != RT_ERR_USER) return 1;\n"
        "  if (rt_create(0, 0) != RT_ERR_USER) return 2;\n"
        "  if (rt_split_dgemm_noalloc(0, 8, 8, 0, 0, 0, 5, 0) != RT_ERR_USER) return 3;\n"
        "  (void)ctx; puts(\"ok\"); return 0;\n}\n")
    exe = tmp_path / "caller"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir,
                        "-lrotran_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
