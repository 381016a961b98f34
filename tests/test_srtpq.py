"""The MPI version's pq-sorted integral files SRTPQIL[.r]/SRTPQLN[.r]
(getpq.F, rotran.par.F:430-506) parsed by rt_srtpq_scan: no GPU needed."""

import collections
import os
import struct

import numpy as np
import pytest

from molfdir_gb300 import fortio, rotran, synth


def summed(cls, its, nts, v, l2, l1):
    """(class, type, label2, label1) -> summed value."""
    out = collections.defaultdict(float)
    c = np.repeat(cls, nts)
    t = np.repeat(its, nts)
    for key in zip(c.tolist(), t.tolist(), l2.tolist(), l1.tolist(), v.tolist()):
        out[key[:4]] += key[4]
    return out


@pytest.mark.parametrize("nranks,nbuf,split", [(1, 256, 0), (3, 16, 5), (4, 7, 3)])
def test_scan_returns_the_serial_integrals(tmp_path, nranks, nbuf, split):
    p = synth.make_problem(5, 7, 3, seed=2)
    fortio.write_srtpq_files(p, str(tmp_path), nranks=nranks, nbuf=nbuf, split_every=split,
                             breit_pairs=3, seed=nranks)
    got = rotran.srtpq_scan(str(tmp_path), nranks, p.n, p.model.n_l)
    want = summed(*p.flat_records())
    have = summed(*got)
    assert set(have) == set(want)
    for k, x in want.items():
        assert have[k] == x, k  # halves of a value add back exactly
    # one record per (class, type); label1 is a stream's pq pair, p >= q
    assert len(set(zip(got[0].tolist(), got[1].tolist()))) == got[0].size
    l1 = got[5]
    assert np.all((l1 >> 16) >= (l1 & 0xFFFF))


def test_scan_irrep_blocks(tmp_path):
    p = synth.make_spinor_problem(6, 10, 4, seed=3, n_irrep=4)
    fortio.write_srtpq_files(p, str(tmp_path), nranks=2, nbuf=32)
    got = rotran.srtpq_scan(str(tmp_path), 2, p.n, p.model.n_l)
    assert summed(*got) == summed(*p.flat_records())


def test_types_follow_inttyp_with_the_larger_pair_first(tmp_path):
    p = synth.make_problem(4, 6, 2, seed=4)
    fortio.write_srtpq_files(p, str(tmp_path), nbuf=64)
    cls, its, nts, v, l2, l1 = rotran.srtpq_scan(str(tmp_path), 1, p.n, p.model.n_l)
    t = np.repeat(its, nts)
    a, b, c, d = l2 >> 16, l2 & 0xFFFF, l1 >> 16, l1 & 0xFFFF
    first = (a > c) | ((a == c) & (b >= d))
    ref = np.where(first, synth.inttyp(a, b, c, d), synth.inttyp(c, d, a, b))
    assert np.array_equal(t, ref)


def test_empty_files(tmp_path):
    with open(tmp_path / "SRTPQIL", "wb"):
        pass
    with open(tmp_path / "SRTPQLN", "wb") as f:
        fortio.write_record(f, struct.pack("<6i", 0, 3084, 1, 3, 4, 7))
    got = rotran.srtpq_scan(str(tmp_path), 1, 7, 3)
    assert got[0].size == 0 and got[3].size == 0


def write_one(tmp_path, recs, irecl=12 + 12 * 4, n=6, nl=3, lrecco=None):
    with open(tmp_path / "SRTPQIL", "wb") as f:
        for ipql, nt, inxt, vals, labs in recs:
            rec = struct.pack("<iii", ipql, nt, inxt)
            rec += np.asarray(vals, "<f8").tobytes() + np.asarray(labs, "<i4").tobytes()
            f.write(rec + b"\0" * (irecl - len(rec)))
    with open(tmp_path / "SRTPQLN", "wb") as f:
        fortio.write_record(f, struct.pack("<6i", len(recs) if lrecco is None else lrecco,
                                           irecl, 1, nl, nl + 1, n))


def pq(p, q):
    return p * (p - 1) // 2 + q


def lab(r, s):
    return (r << 16) | s


def scan_error(tmp_path, n=6, nl=3, nranks=1):
    with pytest.raises(rotran.RotranError) as e:
        rotran.srtpq_scan(str(tmp_path), nranks, n, nl)
    return e.value.code, str(e.value)


def test_chain_links_and_breit_records(tmp_path):
    # stream (2,1): records 1 <- 3; stream (5,4): record 2; Breit (4,2): record 4
    write_one(tmp_path, [(pq(2, 1), 2, 0, [1.0, 2.0], [lab(2, 2), lab(3, 1)]),
                         (pq(5, 4), 1, 0, [3.0], [lab(6, 5)]),
                         (pq(2, 1), 1, 1, [4.0], [lab(3, 3)]),
                         (pq(4, 2), 2, 0, [9.0, 9.0], [lab(5, 1), lab(6, 2)])])
    cls, its, nts, v, l2, l1 = rotran.srtpq_scan(str(tmp_path), 1, 6, 3)
    assert sorted(v.tolist()) == [1.0, 2.0, 3.0, 4.0]
    c = dict(zip(v.tolist(), np.repeat(cls, nts).tolist()))
    assert c == {1.0: 1, 2.0: 1, 4.0: 1, 3.0: 3}


@pytest.mark.parametrize("case,code,text", [
    ("link_other_stream", 2, "broken record chain"),
    ("link_forward", 2, "broken record chain"),
    ("two_links", 2, "broken record chain"),
    ("nt_too_big", 2, "bad record header"),
    ("label_range", 2, "label outside"),
    ("mixed_pair", 2, "mixed L/S label pair"),
    ("short_file", 1, "READ ERROR"),
])
def test_malformed_files(tmp_path, case, code, text):
    good = (pq(2, 1), 1, 0, [1.0], [lab(2, 1)])
    recs = {
        "link_other_stream": [good, (pq(3, 1), 1, 1, [1.0], [lab(3, 3)])],
        "link_forward": [(pq(2, 1), 1, 2, [1.0], [lab(2, 1)]), good],
        "two_links": [good, (pq(2, 1), 1, 1, [1.0], [lab(2, 2)]), (pq(2, 1), 1, 1, [1.0], [lab(3, 2)])],
        "nt_too_big": [(pq(2, 1), 5, 0, [1.0] * 4, [lab(2, 1)] * 4)],
        "label_range": [(pq(2, 1), 1, 0, [1.0], [lab(7, 1)])],
        "mixed_pair": [(pq(2, 1), 1, 0, [1.0], [lab(4, 1)])],
        "short_file": [good],
    }[case]
    if case == "nt_too_big":
        write_one(tmp_path, recs, irecl=12 + 12 * 5)
        with open(tmp_path / "SRTPQLN", "wb") as f:  # the file claims 4 entries per record
            fortio.write_record(f, struct.pack("<6i", 1, 12 + 12 * 4, 1, 3, 4, 6))
    else:
        write_one(tmp_path, recs, lrecco=2 if case == "short_file" else None)
    got_code, msg = scan_error(tmp_path)
    assert got_code == code
    assert text in msg


def test_missing_rank_and_ranges(tmp_path):
    p = synth.make_problem(3, 4, 2, seed=1)
    fortio.write_srtpq_files(p, str(tmp_path), nranks=2, nbuf=8)
    code, msg = scan_error(tmp_path, p.n, p.model.n_l, nranks=3)
    assert code == 1 and "SRTPQLN.2" in msg and "MISSING" in msg
    code, msg = scan_error(tmp_path, p.n, p.model.n_l + 1, nranks=2)
    assert code == 2 and "NSC1" in msg


def test_capacity_protocol(tmp_path):
    p = synth.make_problem(3, 4, 2, seed=1)
    fortio.write_srtpq_files(p, str(tmp_path), nbuf=8)
    lib = rotran.load()
    import ctypes as C
    nrec, nint = C.c_longlong(-1), C.c_longlong(-1)
    rc = lib.rt_srtpq_scan(os.fsencode(str(tmp_path)), 1, p.n, p.model.n_l, 0, C.byref(nrec),
                           C.byref(nint), None, None, None, None, None, None)
    assert rc == rotran.RT_ERR_DIM
    assert nint.value == p.flat_records()[3].size
    assert 1 <= nrec.value <= 42


def test_scan_property_over_random_layouts():
    """Any rank count, record size, repeat pattern and number of Breit
    streams: the parse returns exactly the serial integrals."""
    import tempfile
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=25, deadline=None, derandomize=True)
    @hyp.given(nl=st.integers(1, 5), ns=st.integers(1, 6), seed=st.integers(0, 1000),
               nranks=st.integers(1, 5), nbuf=st.integers(1, 40), split=st.integers(0, 4),
               breit=st.integers(0, 3))
    def prop(nl, ns, seed, nranks, nbuf, split, breit):
        p = synth.make_problem(nl, ns, 1, seed=seed)
        with tempfile.TemporaryDirectory() as d:
            fortio.write_srtpq_files(p, d, nranks=nranks, nbuf=nbuf, split_every=split,
                                     breit_pairs=breit, seed=seed)
            got = rotran.srtpq_scan(d, nranks, p.n, p.model.n_l)
        want = summed(*p.flat_records())
        have = summed(*got)
        assert set(have) == set(want)
        for k, x in want.items():
            assert have[k] == x

    prop()
