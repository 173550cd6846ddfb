"""Dissolving small bins and recruiting leftover / small contigs: the
oracle restatement against the reference's own block (compiled here from
cuda/Cuda2.cu:2064-2283; tests/golden/make_recruit_golden.py) on four seeded
cases, with the reference's verbose flag off and on."""
import os

import numpy as np
import pytest

from oracle import oracle

G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "recruit_golden.npz")


@pytest.mark.parametrize("name", ["a", "b", "c", "d"])
@pytest.mark.parametrize("verbose", [0, 1])
def test_oracle_equals_reference_block(name, verbose):
    z = np.load(G)
    ssz = z[f"{name}_small_sizes"]
    out, sout, st = oracle.recruit(z[f"{name}_abd"], z[f"{name}_small"], z[f"{name}_label"], z[f"{name}_sizes"], ssz,
                                   int(z[f"{name}_min_cls"][0]), int(ssz.sum()) if verbose else 0)
    assert np.array_equal(out, z[f"{name}_out_v{verbose}"])
    assert np.array_equal(sout, z[f"{name}_small_out_v{verbose}"])
    assert st["leftovers"] > 0
