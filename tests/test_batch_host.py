"""Host-side logic of the batched API, without a GPU: how solve_structures groups problems into
shape groups and chunks (the groups are what it deals to its CUDA streams), and the workspace
cache that gives every (slot, stream) its own buffer."""
import numpy as np

from khepri_gb300 import autotune, batch, engine, workloads


def test_shape_groups_cover_every_problem_once():
    ents = [(s.pw, s.layers, s.stack) for s, _, _ in workloads.uneven_structures(24, seed=3, n_pix=16)]
    which = np.arange(len(ents))
    groups, digests = batch._group_plan(ents, which, chunk=None)
    seen = np.concatenate([idx for _, chunks in groups for idx in chunks])
    assert sorted(seen.tolist()) == list(range(len(ents)))
    for key, chunks in groups:
        pw, kinds = key[0], key[1]
        nslots = len({s for k, s in zip(kinds, key[2]) if k == 1}) or 1
        step = autotune.chunk_for(2 * pw[0] * pw[1], nslots)
        assert all(len(idx) <= step for idx in chunks)
        for idx in chunks:
            for p in idx:  # every member has the group's harmonics and layer kinds
                pw_p, layers, stack = ents[which[p]]
                assert tuple(pw_p) == pw
                assert tuple(1 if layers[name][0] == "pixmap" else 0 for name in stack) == tuple(kinds)
    assert len(digests) == len(ents)


def test_explicit_chunk_splits_a_group():
    s = workloads.inverse_design(3, seed=0)[1]
    ents = [(x.pw, x.layers, x.stack) for x in s]
    which = np.repeat(np.arange(3), 5)  # 15 problems over 3 designs of one shape
    groups, _ = batch._group_plan(ents, which, chunk=4)
    assert len(groups) == 1  # same harmonics, kinds, uniform media and map sharing
    sizes = [len(idx) for idx in groups[0][1]]
    assert sizes == [4, 4, 4, 3]


def test_workspace_per_slot_and_growth():
    a = engine.workspace(1000, "cpu", slot=101)
    b = engine.workspace(500, "cpu", slot=101)
    assert b.data_ptr() == a.data_ptr()  # large enough: reused
    c = engine.workspace(500, "cpu", slot=102)
    assert c.data_ptr() != a.data_ptr()  # another slot: its own buffer
    d = engine.workspace(4000, "cpu", slot=101)
    assert d.numel() >= 4000 and engine.workspace(10, "cpu", slot=101).data_ptr() == d.data_ptr()
