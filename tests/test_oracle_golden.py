"""The oracle (C restatement) against fixtures produced by the reference's own
CPU solver: shooter trace, per-slot state and .fin bytes, bit for bit."""
import hashlib

import numpy as np
import pytest

import runner
from helpers import golden, golden_index, same_bits, sha256_file, write_case

CASES = sorted(golden_index())


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(built, workdir, name):
    tri, argv, idx = write_case(name, workdir)
    assert sha256_file(tri) == idx["tri_sha256"], "scene generator drifted from the fixture"
    out = runner.oracle(tri, argv, fp64=idx["fp64"], adaptive=idx.get("adaptive", False))
    g = golden(name)
    assert np.array_equal(runner.trace_array(out["trace"], idx["P"]), g["trace"])
    d = out["dump"]
    assert d["n"] == idx["n_slots"]
    for k in ("parent", "p", "accB", "deltaB", "nb"):
        assert same_bits(d[k], g[k]), k
    assert hashlib.sha256(out["fin"]).hexdigest() == idx["fin_sha256"]
