"""The product's host code (no GPU needed): the compiled ghost fills and the
quadtree's admesh, against the oracle's sequential restatement."""
import numpy as np
import pytest

from oracle import pyoracle as P
from parity_util import oracle_kw
from shim import admesh, ghost_apply, ghost_apply_fused, host_pool, last_by_block, tree_check

GHOST_CASES = [("BWx", "MC", 4, 2, 3), ("rotor", "MC", 5, 2, 30), ("BWx", "WENO5", 3, 4, 10),
               ("rotor", "WENO5", 3, 4, 25)]


@pytest.mark.parametrize("ic,lim,L,ng,steps", GHOST_CASES)
def test_ghost_program_matches_sequential_fill(ic, lim, L, ng, steps):
    o = P.Oracle(ic=ic, limiter=lim, flux="RUSA", cfl=0.4, maxlevs=L, nghosts=ng).init()
    for _ in range(steps):
        o.step()
    st = o.state()
    n = 16 + 2 * ng
    rng = np.random.default_rng(steps)
    for kind, nv in [(0, 8), (1, 2), (1, 8), (2, 1)]:
        f = rng.standard_normal((st["lastActive"], nv, n, n))
        ref = o.fill(f, kind)
        got, nops, _ = ghost_apply(st, kind, nv, f, L, ng)
        assert nops > 0
        assert np.array_equal(ref, got), (kind, nv, int((ref != got).sum()))
        # grouped by block (checked inside the shim), all in leaves: the fills
        # can run inside the step's per-block kernels
        assert last_by_block() == 1


@pytest.mark.parametrize("ic,lim,L,ng,steps", GHOST_CASES)
def test_fused_fill_order_free(ic, lim, L, ng, steps):
    """The fill as the fused kernels apply it (all snapshots first, then each
    block's gathers in place, blocks in any order) equals the sequential walk:
    no gather reads a cell that another block's gathers write."""
    o = P.Oracle(ic=ic, limiter=lim, flux="RUSA", cfl=0.4, maxlevs=L, nghosts=ng).init()
    for _ in range(steps):
        o.step()
    st = o.state()
    n = 16 + 2 * ng
    rng = np.random.default_rng(steps + 7)
    for kind, nv in [(0, 8), (1, 2), (2, 1)]:
        f = rng.standard_normal((st["lastActive"], nv, n, n))
        ref = o.fill(f, kind)
        for seed in (1, 2, 3):
            assert np.array_equal(ghost_apply_fused(st, kind, nv, f, L, seed, ng), ref), (kind, seed)


@pytest.mark.parametrize("seed,periodic", [(11, False), (12, False), (13, True)])
def test_ghost_program_on_random_mark_trees(seed, periodic):
    """The compiled ghost fills equal the oracle's sequential fills on trees
    remeshed by random marks (coarse / fine layouts no run of the
    reference's criterion produces), every fill kind."""
    kw = dict(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=5)
    nroots = (2, 2)
    if periodic:
        kw = dict(ic="OT", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=4, nroots=(3, 3), periodic=True,
                  geom_ref=False, lenx=2 * np.pi, leny=2 * np.pi)
        nroots = (3, 3)
    L = kw["maxlevs"]
    o = P.Oracle(**kw).init()
    o.set_remesh(False)
    rng = np.random.default_rng(seed)
    for it in range(8):
        n = o.info()["lastActive"]
        o.admesh_marked(rng.random(n) < 0.15, rng.random(n) < 0.5)
        st = o.state()
        assert tree_check(st, L, 2, nroots, periodic) is None
        for kind, nv in [(0, 8), (1, 2), (2, 1)]:
            f = rng.standard_normal((st["lastActive"], nv, 20, 20))
            got, _, _ = ghost_apply(st, kind, nv, f, L, 2, nroots, periodic)
            ref = o.fill(f, kind)
            assert np.array_equal(ref, got), (it, kind)
            assert last_by_block() == 1
            assert np.array_equal(ghost_apply_fused(st, kind, nv, f, L, seed + it, 2, nroots, periodic), ref)


def test_ghost_program_periodic_16_roots():
    o = P.Oracle(ic="OT", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=3, nroots=(4, 4), periodic=True,
                 geom_ref=False, lenx=2 * np.pi, leny=2 * np.pi).init()
    for _ in range(3):
        o.step()
    st = o.state()
    f = np.random.default_rng(1).standard_normal((st["lastActive"], 8, 20, 20))
    got, _, _ = ghost_apply(st, 0, 8, f, 3, 2, (4, 4), True)
    assert np.array_equal(o.fill(f, 0), got)


@pytest.mark.parametrize("ic,flux,L,steps", [("rotor", "RUSA", 5, 40), ("BWx", "RUSA", 4, 12)])
def test_admesh_matches_oracle(ic, flux, L, steps):
    o = P.Oracle(ic=ic, limiter="MC", flux=flux, cfl=0.4, maxlevs=L).init()
    o.set_remesh(False)
    changes = 0
    for _ in range(steps):
        o.step()
        st = o.state()
        grad = P.criteria_grad(o.get("W"))
        got, nr, nc = admesh(st, grad, L)
        o.admesh()
        ref = o.state()
        changes += nr + nc
        assert got["lastActive"] == ref["lastActive"]
        assert np.array_equal(got["leafs"], ref["leafs"])
        assert np.array_equal(got["lp"], ref["lp"])
        assert np.array_equal(got["icoord"], ref["icoord"])
        assert got["nbleafs"] == ref["nbleafs"]
    assert changes > 0


def _leaf_rects(st, L):
    """Leaves as [level, x0, y0, size] in cells of the finest level."""
    lf = np.flatnonzero(st["leafs"])
    lev = st["lp"][lf, 0]
    scale = 2 ** (L - 1 - lev)
    return lev, st["icoord"][lf, 0] * scale, st["icoord"][lf, 1] * scale, 16 * scale


def _max_level_jump(st, L):
    """Largest level difference between two leaves sharing an edge."""
    lev, x0, y0, sz = _leaf_rects(st, L)
    x1, y1 = x0 + sz, y0 + sz
    ov_y = (np.minimum(y1[:, None], y1[None]) - np.maximum(y0[:, None], y0[None])) > 0
    ov_x = (np.minimum(x1[:, None], x1[None]) - np.maximum(x0[:, None], x0[None])) > 0
    touch = ((x1[:, None] == x0[None]) & ov_y) | ((y1[:, None] == y0[None]) & ov_x)
    return int(np.abs(lev[:, None] - lev[None])[touch].max())


def test_admesh_marked_with_criteria_marks_is_admesh():
    """Tree::admesh_marked given criteria.cpp's flags gives Tree::admesh's
    tree, step after step of a rotor run."""
    L = 5
    o = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=L).init()
    o.set_remesh(False)
    changes = 0
    for _ in range(30):
        o.step()
        st = o.state()
        grad = P.criteria_grad(o.get("W"))
        marks = P.criteria_flags(grad, st["leafs"], st["lp"][:, 0], L)
        a, nr, nc = admesh(st, grad, L)
        b, mr, mc = admesh(st, None, L, marks=marks)
        assert (nr, nc) == (mr, mc)
        for k in ("lastActive", "nbleafs"):
            assert a[k] == b[k]
        for k in ("leafs", "lp", "icoord"):
            assert np.array_equal(a[k], b[k])
        o.admesh()
        changes += nr + nc
    assert changes > 0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_admesh_marked_random_marks_keep_the_tree_balanced(seed):
    """Arbitrary marks: the neighbour rules keep leaves that share an edge
    within one level; refining adds three leaves, coarsening removes three,
    marks on the finest level or on non-leaves change nothing, and coarsening
    needs all four siblings marked."""
    L = 5
    o = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=L).init()
    st = o.state()
    rng = np.random.default_rng(seed)
    total = np.zeros(2, int)
    for it in range(14):
        n = st["lastActive"]
        iref = rng.random(n) < (0.08 if it < 9 else 0.0)   # grow, then mostly coarsen
        ico = rng.random(n) < (0.6 if it < 9 else 0.95)
        got, nr, nc = admesh(st, None, L, marks=(iref, ico))
        total += (nr, nc)
        assert tree_check(got, L) is None, (it, tree_check(got, L))
        assert got["leafs"].sum() == st["leafs"].sum() + 3 * nr - 3 * nc
        assert got["nbleafs"] == st["nbleafs"] + 4 * nr - 3 * nc
        assert _max_level_jump(got, L) <= 1
        # every coarsened dad had four leaf sons marked for coarsening (a
        # block that turns leaf because its father was refined, son-ID
        # reuse, is not a coarsened dad)
        m = got["lastActive"]
        for d in np.flatnonzero(got["leafs"][:n] & ~st["leafs"][:n]):
            father = st["lp"][d, 1]
            if father >= 0 and st["leafs"][father]:
                continue
            s0 = st["lp"][d, 2]
            sons = [s0, st["lp"][s0, 5], st["lp"][s0, 7], st["lp"][st["lp"][s0, 7], 5]]
            assert all(st["leafs"][q] and ico[q] and not iref[q] for q in sons)
        assert m >= n
        st = got
    assert total[0] > 20 and total[1] > 20, total
    # marks on the finest level (refine) and on non-leaves change nothing
    n = st["lastActive"]
    fine = st["leafs"] & (st["lp"][:, 0] == L - 1)
    same, nr, nc = admesh(st, None, L, marks=(fine | ~st["leafs"], ~st["leafs"]))
    assert (nr, nc) == (0, 0)
    assert np.array_equal(same["lp"], st["lp"]) and same["lastActive"] == n


def test_admesh_marked_matches_oracle_on_random_marks():
    """The product's Tree::admesh_marked and the oracle's marked admesh give
    the same tree for the same arbitrary marks; the oracle's marked admesh
    with criteria.cpp's flags is its own admesh (tree and fields)."""
    L = 5
    o = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=L).init()
    o.set_remesh(False)
    rng = np.random.default_rng(7)
    for it in range(10):
        o.step()
        st = o.state()
        n = st["lastActive"]
        iref, ico = rng.random(n) < 0.06, rng.random(n) < 0.7
        got, _, _ = admesh(st, None, L, marks=(iref, ico))
        o.admesh_marked(iref, ico)
        ref = o.state()
        assert got["lastActive"] == ref["lastActive"] and got["nbleafs"] == ref["nbleafs"]
        for k in ("leafs", "lp", "icoord"):
            assert np.array_equal(got[k], ref[k]), (it, k)
    a = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=L).init()
    b = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=L).init()
    for x in (a, b):
        x.set_remesh(False)
        for _ in range(6):
            x.step()
    st = a.state()
    marks = P.criteria_flags(P.criteria_grad(a.get("W")), st["leafs"], st["lp"][:, 0], L)
    a.admesh()
    b.admesh_marked(*marks)
    sa, sb = a.state(), b.state()
    assert sa["lastActive"] > st["lastActive"]
    for k in ("leafs", "lp", "icoord", "U", "Bi"):
        assert np.array_equal(sa[k], sb[k]), k


TREE_RUNS = [(dict(ic="rotor", flux="HLLD", maxlevs=4), 60, (2, 2), False),
             (dict(ic="rotor", flux="RUSA", maxlevs=5), 120, (2, 2), False),
             (dict(ic="BWx", flux="RUSA", maxlevs=4), 120, (2, 2), False),
             (dict(ic="OT", flux="RUSA", maxlevs=3, nroots=(4, 4), periodic=True, geom_ref=False,
                   lenx=2 * np.pi, leny=2 * np.pi), 40, (4, 4), True)]


@pytest.mark.parametrize("kw,steps,nroots,periodic", TREE_RUNS)
def test_tree_check_accepts_every_tree_admesh_builds(kw, steps, nroots, periodic):
    """Tree::check (run on trees handed in by amr_set_tree) passes every
    tree of these runs, step by step, refinement and coarsening included."""
    o = P.Oracle(limiter="MC", cfl=0.4, **kw).init()
    L = kw["maxlevs"]
    seen = set()
    for k in range(steps + 1):
        st = o.state()
        assert tree_check(st, L, 2, nroots, periodic) is None, (k, tree_check(st, L, 2, nroots, periodic))
        seen.add(st["lastActive"])
        o.step()
    assert len(seen) > 1


def test_tree_check_accepts_blast_and_kh_trees():
    """The seeded blast instances (uneven levels, as checkpointed in a batch)
    and the single-level periodic KH problem pass Tree::check step by step."""
    import amr2d_mhd_gb300 as amr
    cfgs = [amr.blast_config(3, i) for i in range(3)] + [amr.kh_config(42)]
    for c in cfgs:
        c.maxlevs = min(c.maxlevs, 4)
        o = P.Oracle(**oracle_kw(c, 4)).init()
        for k in range(26):
            msg = tree_check(o.state(), c.maxlevs, c.nghosts, (c.nroots_x, c.nroots_y), bool(c.periodic))
            assert msg is None, (c.ic, k, msg)
            o.step()


def test_tree_check_rejects_broken_trees():
    """IDs out of range, broken father / son or sibling links, neighbours
    outside the active tree and unbalanced neighbours are all refused."""
    L = 5
    o = P.Oracle(ic="rotor", limiter="MC", flux="RUSA", cfl=0.4, maxlevs=L).init()
    o.run(40)
    st = o.state()
    assert tree_check(st, L) is None
    lp, lf = st["lp"], st["leafs"]
    n = st["lastActive"]
    leaf = int(np.flatnonzero(lf & (lp[:, 0] >= 2))[0])
    dad = int(np.flatnonzero(~lf[:n] & (lp[:n, 2] != 0) & (lp[:n, 0] >= 1))[0])

    def broken(edit):
        bad = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in st.items()}
        edit(bad)
        return tree_check(bad, L)

    def setlp(b, c, v):
        return lambda t: t["lp"].__setitem__((b, c), v)

    assert "neighbour ID" in broken(setlp(leaf, 5, n))
    assert "neighbour ID" in broken(setlp(leaf, 4, -2))
    assert "father ID" in broken(setlp(leaf, 1, n + 7))
    assert "first-son ID" in broken(setlp(dad, 2, n - 2))
    assert "level" in broken(setlp(leaf, 0, L))
    assert "sibling number" in broken(setlp(leaf, 3, 4))
    assert "father" in broken(setlp(leaf, 3, (lp[leaf, 3] + 1) % 4))
    s0 = lp[dad, 2]
    assert "links between its sons" in broken(setlp(s0, 5, s0 + 2))
    assert "roots" in broken(setlp(0, 0, 1))
    assert "a leaf whose father is a leaf" in broken(lambda t: t["leafs"].__setitem__(lp[leaf, 1], True))
    # a neighbour pointer to a block two levels coarser
    coarse = int(np.flatnonzero(lp[:n, 0] == lp[leaf, 0] - 2)[0])
    assert broken(setlp(leaf, 4, coarse)) is not None
    assert "last_active" in broken(lambda t: t.__setitem__("lastActive", 3))


@pytest.mark.parametrize("threads", [1, 2, 8])
def test_host_pool_parallel_loops(threads):
    """The engine's persistent host threads (remesh, compile and layout loops
    of a batch): 300 consecutive loops of 1000 items, every item once."""
    assert host_pool(300, 1000, threads) == 0
