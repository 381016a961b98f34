"""Regenerate tests/golden/oracle_n14_k4.npz.

The record structure (which MDCINT records and elements exist) comes from
the oracle's restatement of OUTPP1/OUTPP2/PPSYM; the values stored are the
independent dense four-index sums for those elements, so the fixture pins
both the structure and the values of a seeded 14-function, 4-pair case.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import pyoracle  # noqa: E402
from molfdir_gb300 import synth  # noqa: E402
from test_oracle import dense_full, spinor_of  # noqa: E402

p = synth.make_problem(6, 8, 4, seed=11)
img = pyoracle.run(p)
v = dense_full(p)
dense_val = np.empty_like(img.val)
off = 0
for a, b, nz in img.hdr:
    for z in range(nz):
        c, d = img.idx[off + z]
        dense_val[off + z] = v[spinor_of(p, a), spinor_of(p, b), spinor_of(p, c), spinor_of(p, d)]
    off += nz
np.savez_compressed(os.path.join(HERE, "oracle_n14_k4.npz"), hdr=img.hdr, idx=img.idx,
                    dense_val=dense_val)
print("wrote", img.hdr.shape[0], "records,", img.idx.shape[0], "elements")
