"""Batched transforms (rt_batch_*): grouped GEMM launches over many contexts,
tuned tile widths, CUDA-graph replay; results must equal each context's own
rt_transform bit for bit (needs a GB300)."""

import numpy as np
import pytest

from molfdir_gb300 import rotran, synth

pytestmark = pytest.mark.gpu

SIZES = [(5, 7, 3, 1), (8, 12, 6, 2), (3, 5, 2, 3), (10, 14, 8, 4), (6, 9, 4, 5), (4, 6, 5, 6)]


def make_ctx(prob, precision=rotran.RT_PREC_SPLIT_BF16):
    rt = rotran.Rotran.for_problem(prob, precision=precision)
    rt.set_problem_coefficients(prob)
    rt.add_problem_records(prob)
    return rt


def problems(n_irrep=1):
    return [synth.make_problem(nl, ns, nkr, seed=s, n_irrep=n_irrep) for nl, ns, nkr, s in SIZES]


@pytest.mark.parametrize("n_irrep", [1, 4])
def test_batch_equals_single_transforms(n_irrep):
    probs = problems(n_irrep)
    ref = []
    for p in probs:
        rt = make_ctx(p)
        rt.transform()
        ref.append(rt.result())
        rt.close()
    rts = [make_ctx(p) for p in probs]
    with rotran.Batch(rts) as b:
        for rep in range(3):  # tuning + capture, then two graph replays
            b.run()
            for rt, (h, i, v) in zip(rts, ref):
                h2, i2, v2 = rt.result()
                assert np.array_equal(h, h2) and np.array_equal(i, i2)
                assert np.array_equal(v, v2)
        st = b.stats()
        print(st.as_dict())
        assert st.instances == len(probs)
        assert st.grouped_launches >= 4 and st.tile128 + st.tile64 == st.grouped_launches
        assert st.graph_nodes >= st.kernel_launches > 0
    for rt in rts:
        rt.close()


def test_batch_matches_oracle():
    import pyoracle
    from util import compare_streams
    probs = problems()[:3]
    rts = [make_ctx(p) for p in probs]
    with rotran.Batch(rts) as b:
        b.run()
        for rt, p in zip(rts, probs):
            img = pyoracle.run(p)
            assert compare_streams(rt.result(), (img.hdr, img.idx, img.val), 1e-10) <= 1e-10
    for rt in rts:
        rt.close()


def test_batch_rejects_changed_inputs():
    probs = problems()[:2]
    rts = [make_ctx(p) for p in probs]
    b = rotran.Batch(rts)
    b.run()
    rts[1].add_problem_records(probs[1])  # records added after the batch was built
    with pytest.raises(rotran.RotranError) as ei:
        b.run()
    assert ei.value.code == 5
    b.close()
    for rt in rts:
        rt.close()


def test_batch_needs_split_precision():
    p = problems()[0]
    rt = make_ctx(p, precision=rotran.RT_PREC_FP64)
    with pytest.raises(rotran.RotranError):
        rotran.Batch([rt])
    rt.close()


def test_tile_width_cache(tmp_path, monkeypatch):
    """RT_TUNE_CACHE: the first batch times both tile widths per grouped stage
    and writes its choices under each stage's shape class; a later batch of
    the same shapes takes them from the file without tuning runs (ms_tune 0)
    and gives the same results."""
    path = tmp_path / "tune.json"
    monkeypatch.setenv("RT_TUNE_CACHE", str(path))
    probs = problems()
    outs = []
    for attempt in range(2):
        rts = [make_ctx(p) for p in probs]
        with rotran.Batch(rts) as b:
            b.run()
            st = b.stats()
            outs.append([rt.result() for rt in rts])
        for rt in rts:
            rt.close()
        if attempt == 0:
            assert st.ms_tune > 0.0
            text = path.read_text()
            assert text.count(":") >= 2 * (st.tile64 + st.tile128)
        else:
            assert st.ms_tune == 0.0
    for a, b_ in zip(*outs):
        for x, y in zip(a, b_):
            assert np.array_equal(x, y)
