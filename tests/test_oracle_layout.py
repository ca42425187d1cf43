"""CPU checks of the sort-contract restatement (oracle/layout.py) that the
GPU layout test compares against: its prediction reproduces the reference's
predicted positions bit for bit, its grid matches the library's own mirror
of the table choice (fluidsim.simulation.key_table), and its order and start
table are consistent (every particle once, keys ascending, cells contiguous
inside a key, start = exclusive prefix of the key counts)."""
import numpy as np
import pytest

from conftest import fixture_params, load_fixture, substep_fixtures


@pytest.mark.parametrize("name", substep_fixtures())
def test_predict_matches_reference(name):
    from oracle import layout
    fx = load_fixture(name)
    p = fixture_params(fx)
    assert np.array_equal(layout.predict(p, fx["pos_in"], fx["vel_in"], fx["dt"]), fx["pred"])


@pytest.mark.parametrize("table", [0, 1, 2])
@pytest.mark.parametrize("name", substep_fixtures())
def test_layout_consistent(name, table):
    from fluidsim.simulation import key_table
    from oracle import layout
    fx = load_fixture(name)
    p = fixture_params(fx)
    n = fx["pred"].shape[0]
    L = layout.sort_layout(p, fx["pred"], table)
    assert (L["direct"], L["start"].shape[0] - 1) == key_table(p, n, table)
    s = L["slot_ids"]
    assert np.array_equal(np.sort(s), np.arange(n, dtype=np.uint32))
    ks, cs = L["key"][s].astype(np.int64), L["cell"][s].astype(np.int64)
    assert np.all(np.diff(ks) >= 0)
    same = np.diff(ks) == 0
    assert np.all(np.diff(cs)[same] >= 0)  # cells ascend inside a key
    ids_same_cell = same & (np.diff(cs) == 0)
    assert np.all(np.diff(s.astype(np.int64))[ids_same_cell] > 0)  # then caller index
    st = L["start"].astype(np.int64)
    assert st[0] == 0 and st[-1] == n and np.all(np.diff(st) >= 0)
    for slot in range(n):
        k = ks[slot]
        assert st[k] <= slot < st[k + 1]
    if L["direct"]:
        assert np.array_equal(L["key"], L["cell"])
    else:
        assert np.array_equal(L["key"], L["cell"] % np.uint32(n))


@pytest.mark.parametrize("name", substep_fixtures())
def test_reference_lookup_matches_reference(name):
    """The numpy restatement of the reference's own lookup (hash, key,
    (key, index) order, startIndices) reproduces the reference's outputs."""
    from oracle import layout
    fx = load_fixture(name)
    p = fixture_params(fx)
    L = layout.reference_lookup(fx["pred"], np.float32(p.radius))
    for k in ("hash", "key", "sorted_ids", "start"):
        assert np.array_equal(L[k], fx[k]), k
