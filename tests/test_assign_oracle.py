"""The oracle of the equal-size group assignment (oracle/assign_oracle.cpp,
restating EMAN2's Util::assign_groups as bin/sp_isac2_gpu.py:1114-1136 calls
and reads it).  EMAN2 is not vendored with the reference, so no golden output
of Util::assign_groups exists here: the oracle is pinned by hand-worked
cases, by a second, independent restatement of the host loop in Python, by
the caller's own reading of the list (bin/sp_isac2_gpu.py:1121-1136), and by
the properties that define the result (sizes; no particle and group outside
the assignment that rank each other above their own partners)."""
import numpy as np
import pytest


def python_assign(d, nref, nima):
    """The host loop, written out plainly: pairs by (peak desc, index asc)."""
    flat = [float(x) for x in np.asarray(d, np.float32).reshape(-1)]
    order = sorted(range(nref * nima), key=lambda l: (-flat[l], l))
    maxasi, extra = nima // nref, nima % nref
    members = [[] for _ in range(nref)]
    placed, closed = [False] * nima, [False] * nref
    open_, last, b = nref, 0, 0
    while open_:
        while True:
            g, p = divmod(order[b], nima)
            if not placed[p] and not closed[g]:
                break
            b += 1
        members[g].append(p)
        placed[p] = True
        if len(members[g]) >= (maxasi if open_ > 1 else maxasi + extra):
            closed[g] = True
            open_ -= 1
            last = g
    out = [m for g in range(nref) for m in members[g][:maxasi]]
    return out + members[last][maxasi:] + [last]


def pair_rank(d):
    """Position of every pair in the host order (0 = first)."""
    flat = np.asarray(d, np.float32).reshape(-1).astype(np.float64) + 0.0
    order = np.lexsort((np.arange(flat.size), -flat))
    rank = np.empty(flat.size, np.int64)
    rank[order] = np.arange(flat.size)
    return rank


def check_stable(ids, d, nref, nima):
    """Every group holds maxasi core members, the last group the leftovers
    too, and no (group, particle) pair outside the core ranks before both the
    particle's own pair and the group's worst core pair."""
    maxasi, extra = nima // nref, nima % nref
    ids = list(ids)
    assert len(ids) == nima + 1
    assert sorted(ids[:nima]) == list(range(nima))
    last = ids[-1]
    rank = pair_rank(d).reshape(nref, nima)
    own = np.full(nima, np.iinfo(np.int64).max)
    worst = np.zeros(nref, np.int64)
    for g in range(nref):
        mem = ids[g * maxasi:(g + 1) * maxasi]
        own[mem] = rank[g, mem]
        worst[g] = rank[g, mem].max()
    # core members in joining order; the last group closes last
    for g in range(nref):
        mem = ids[g * maxasi:(g + 1) * maxasi]
        assert (np.diff(rank[g, mem]) > 0).all()
    assert worst[last] == worst.max()
    left = ids[nref * maxasi:nima]
    assert len(left) == extra
    if extra:
        assert (np.diff(rank[last, left]) > 0).all()
    blocking = (rank < own[None, :]) & (rank < worst[:, None])
    assert not blocking.any()


def test_hand_worked_case(oracle_mod):
    d = np.array([[0.9, 0.8, 0.1, 0.7, 0.2],
                  [0.3, 0.85, 0.6, 0.65, 0.5]], np.float32)
    # (0,p0) (1,p1) [0,p1 skip] (0,p3) closes group 0; (1,p2) (1,p4): the last
    # group takes maxasi + 1 = 3
    ids = oracle_mod.assign_groups(d, 2, 5)
    assert list(ids) == [0, 3, 1, 2, 4, 1]
    assert list(oracle_mod.belongsto_from_id_list(ids, 2, 5)) == [0, 1, 1, 0, 1]


def test_equal_peaks_take_the_smaller_pair_index(oracle_mod):
    assert list(oracle_mod.assign_groups(np.ones((2, 2), np.float32), 2, 2)) == [0, 1, 1]
    # -0.0 and +0.0 are equal peaks
    d = np.array([[-0.0, 0.0, 0.0], [0.0, -0.0, 1.0]], np.float32)
    assert list(oracle_mod.assign_groups(d, 2, 3)) == python_assign(d, 2, 3)


@pytest.mark.parametrize("nref,nima", [(1, 1), (1, 9), (3, 3), (3, 10), (4, 13), (5, 7), (7, 50), (16, 333)])
@pytest.mark.parametrize("kind", ["normal", "ties", "signed"])
def test_oracle_equals_the_plain_loop(oracle_mod, nref, nima, kind):
    rng = np.random.default_rng(nref * 1000 + nima)
    d = rng.normal(size=(nref, nima)).astype(np.float32)
    if kind == "ties":
        d = np.round(d * 2) / 2
    elif kind == "signed":
        d = np.where(rng.random(d.shape) < 0.2, np.float32(-0.0), d)
        d[0, 0] = np.inf
        d[-1, -1] = -np.inf
    ids = oracle_mod.assign_groups(d, nref, nima)
    assert list(ids) == python_assign(d, nref, nima)
    check_stable(ids, d, nref, nima)


def test_caller_reading_matches_the_groups(oracle_mod):
    rng = np.random.default_rng(7)
    nref, nima = 12, 1000          # maxasi 83, 4 leftovers
    d = rng.random((nref, nima), dtype=np.float32)
    ids = oracle_mod.assign_groups(d, nref, nima)
    bel = oracle_mod.belongsto_from_id_list(ids, nref, nima)
    counts = np.bincount(bel, minlength=nref)
    assert sorted(counts.tolist()) == [83] * 11 + [87]
    assert counts[ids[-1]] == 87


def test_oracle_rejects_bad_input(oracle_mod):
    with pytest.raises(ValueError):
        oracle_mod.assign_groups(np.zeros((3, 2), np.float32), 3, 2)      # nima < nref
    d = np.zeros((2, 4), np.float32)
    d[1, 2] = np.nan
    with pytest.raises(ValueError):
        oracle_mod.assign_groups(d, 2, 4)
