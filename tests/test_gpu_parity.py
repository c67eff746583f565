"""GPU step vs the CPU oracle, bit-exact, through the C ABI.

In table mode every decision of the step (normals, cell keys, the in-cell
order, candidate pairs, coins, the matching, product placement) is made by
correctly rounded IEEE operations, so the GPU slot array, the cell starts,
the candidate-pair list and the event counters must equal the oracle's
exactly, step after step.  Positions are compared bit for bit, a stronger
bar than the 1e-5 relative tolerance the step is specified to.
"""
import numpy as np
import pytest

from gpusmoldyn_gb300 import _lib as L
from gpusmoldyn_gb300.configs import rng, uniform_positions
from gpusmoldyn_gb300.system import System
from oracle import py as orc

pytestmark = pytest.mark.gpu


def gpu_records(s):
    xyz, w = s.slots()
    return orc.slots_to_records(xyz, w)


def sort_pairs(p):
    p = np.asarray(p, np.uint32).reshape(-1, 4)
    if len(p) == 0:
        return p
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def run_parity(s, steps, check_cells=True, batch=1):
    o = orc.OracleSystem(s)
    recs = gpu_records(s)
    ev = np.zeros(max(s.n_reactions, 1), np.uint64)
    total_pairs = 0
    t = 0
    while t < steps:
        k = min(batch, steps - t)
        s.step(k)
        s.synchronize()
        for j in range(k):
            res = o.step(t + j, recs, want_cells=check_cells and j == k - 1, want_pairs=j == k - 1, events=ev)
            recs = res["recs"]
        got = gpu_records(s)
        assert got.shape == recs.shape, (t, got.shape, recs.shape)
        bad = np.nonzero(np.any(got != recs, axis=1))[0]
        assert len(bad) == 0, f"step {t + k - 1}: {len(bad)} records differ, first {bad[:5]}"
        if check_cells and o.s.sorted:
            np.testing.assert_array_equal(s.cells(), res["cells"])
        if o.s.sorted:
            gp, op = sort_pairs(s.pairs()), sort_pairs(res["pairs"])
            np.testing.assert_array_equal(gp, op)
            total_pairs += len(op)
        t += k
    np.testing.assert_array_equal(s.event_counts(), ev[:s.n_reactions])
    return recs, total_pairs, ev


def dense_a_b(n_a, n_b, side, seed, normals="table", kon=0.01, **kw):
    s = System((0, 0, 0), (side, side, side), dt=1e-3, seed=seed, normals=normals, **kw)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], kon)
    s.finalize()
    g = rng(seed)
    pos = uniform_positions(g, n_a + n_b, (0, 0, 0), (side, side, side))
    s.set_particles(pos, np.concatenate([np.zeros(n_a), np.ones(n_b)]).astype(np.int32))
    return s


SORTS = ["binned", "compact"]


@pytest.mark.parametrize("sort", SORTS)
def test_irreversible_c1_shape_bit_exact(sort):
    # c1 at a higher rate so that each step has reactions and contested pairs
    s = dense_a_b(2000, 2000, 2.0, seed=11, kon=5.0, sort=sort)
    _, npairs, ev = run_parity(s, 25)
    assert npairs > 100 and ev[0] > 100


def test_contested_pairs_bit_exact():
    # dense enough that particles have several partners: the matching matters
    s = dense_a_b(3000, 3000, 1.2, seed=12, kon=4.0)
    o = orc.OracleSystem(s)
    recs = gpu_records(s)
    res = o.step(0, recs, want_pairs=True)
    s.step(1)
    s.synchronize()
    pairs = res["pairs"]
    assert len(pairs) > 50
    # some particle appears in more than one candidate pair
    ends = np.concatenate([pairs[:, 0], pairs[:, 1]])
    assert np.bincount(ends).max() >= 2
    assert pairs[:, 3].sum() < len(pairs)
    np.testing.assert_array_equal(gpu_records(s), res["recs"])
    np.testing.assert_array_equal(sort_pairs(s.pairs()), sort_pairs(pairs))


def test_reaction_probability_coin_bit_exact():
    s = System((0, 0, 0), (1.5, 1.5, 1.5), dt=1e-3, seed=13, normals="table")
    A, B, Cc, Dd = s.add_species(1.0), s.add_species(0.3), s.add_species(0.5), s.add_species(2.0)
    r = s.add_reaction(2, [A, B], [Cc, Dd], 1.5)  # a ~ 0.09 um
    s.set_reaction_probability(r, 0.35)
    s.set_product_placement(r, L.BD_PP_UNBINDRAD, 0.02)
    s.finalize()
    g = rng(13)
    pos = uniform_positions(g, 6000, (0, 0, 0), (1.5, 1.5, 1.5))
    s.set_particles(pos, (np.arange(6000) % 2).astype(np.int32))
    _, npairs, ev = run_parity(s, 12)
    assert ev[0] > 50


def test_reversible_with_offsets_bit_exact():
    # attainable pgem: both unbinding products are displaced along a random
    # direction and the forward radius is calibrated with that b
    s = System((0, 0, 0), (2.0, 2.0, 2.0), dt=5e-4, seed=14, normals="table")
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 2.0)
    u = s.add_reaction(1, [Cc], [A, B], 200.0)
    s.set_product_placement(u, L.BD_PP_PGEM, 0.02)
    s.finalize()
    assert s.reaction_info(u)["unbind_radius"] > 0
    g = rng(14)
    pos = uniform_positions(g, 6000, (0, 0, 0), (2.0, 2.0, 2.0))
    s.set_particles(pos, (np.arange(6000) % 3).astype(np.int32))
    _, npairs, ev = run_parity(s, 30)
    assert ev[0] > 20 and ev[1] > 20


@pytest.mark.parametrize("sort", SORTS)
def test_mixed_network_bit_exact(sort):
    # zeroth-order births (one and two products), decay, conversion, a
    # displaced two-product birth, a homodimer and a two-product pair reaction
    s = System((0, 0, 0), (3.0, 2.0, 2.5), dt=1e-3, seed=15, normals="table", sort=sort)
    for d in (0.7, 0.3, 2.0, 0.1, 1.2):
        s.add_species(d)
    s.add_reaction(0, [], [0], 300.0)
    s.add_reaction(0, [], [3, 4], 80.0)
    s.add_reaction(1, [0], [1], 5.0)
    s.add_reaction(1, [0], [], 3.0)
    b = s.add_reaction(1, [0], [1, 2], 7.5)
    s.set_product_placement(b, L.BD_PP_UNBINDRAD, 0.05)
    s.add_reaction(2, [2, 2], [3], 2.0)
    s.add_reaction(1, [3], [], 2.0)
    p = s.add_reaction(2, [1, 3], [0, 4], 0.5)
    s.set_product_placement(p, L.BD_PP_UNBINDRAD, 0.03)
    s.add_reaction(2, [4, 0], [], 1.0)
    s.finalize()
    g = rng(15)
    pos = uniform_positions(g, 5000, (0, 0, 0), (3.0, 2.0, 2.5))
    s.set_particles(pos, (np.arange(5000) % 5).astype(np.int32))
    recs, npairs, ev = run_parity(s, 30)
    assert np.all(ev > 0), ev


def test_diffusion_only_in_place_bit_exact():
    s = System((-1, -1, -1), (1, 1, 1), dt=1e-2, seed=16, normals="table")
    s.add_species(0.3)
    s.add_species(0.1)
    s.add_reaction(0, [], [1], 50.0)  # births appended after the slots
    s.finalize()
    g = rng(16)
    pos = uniform_positions(g, 20000, (-1, -1, -1), (1, 1, 1))
    s.set_particles(pos, (np.arange(20000) % 2).astype(np.int32))
    recs, _, ev = run_parity(s, 20, check_cells=False)
    assert recs.shape[0] == 20000 + ev[0]


def test_graph_batches_equal_single_steps():
    a = dense_a_b(1500, 1500, 1.5, seed=17, kon=5.0)
    b = dense_a_b(1500, 1500, 1.5, seed=17, kon=5.0)
    a.step(19)
    a.synchronize()
    for _ in range(19):
        b.step(1)
    b.synchronize()
    np.testing.assert_array_equal(gpu_records(a), gpu_records(b))
    assert a.step_count() == b.step_count() == 19


@pytest.mark.parametrize("sort", SORTS)
def test_capacity_growth_replays_exactly(sort):
    """Births overflow a tight capacity: the step is replayed after the
    buffers grow, giving the same result as a roomy run."""
    def make(cap):
        s = System((0, 0, 0), (2, 2, 2), dt=1e-3, seed=18, normals="table", capacity=cap, sort=sort)
        s.add_species(1.0)
        s.add_species(1.0)
        s.add_reaction(1, [0], [0, 1], 50.0)   # ~5% of the A give birth every step
        s.add_reaction(2, [0, 1], [0], 0.2)
        s.finalize()
        g = rng(18)
        s.set_particles(uniform_positions(g, 4000, (0, 0, 0), (2, 2, 2)), np.zeros(4000, np.int32))
        return s
    tight, roomy = make(4010), make(100000)
    for s in (tight, roomy):
        s.step(40)
        s.synchronize()
    np.testing.assert_array_equal(gpu_records(tight), gpu_records(roomy))
    np.testing.assert_array_equal(tight.event_counts(), roomy.event_counts())
    assert tight.count() > 4010


def test_pair_capacity_growth_replays_exactly():
    a = dense_a_b(3000, 3000, 1.2, seed=19, kon=4.0, pair_capacity=8)
    b = dense_a_b(3000, 3000, 1.2, seed=19, kon=4.0)
    for s in (a, b):
        s.step(5)
        s.synchronize()
    np.testing.assert_array_equal(gpu_records(a), gpu_records(b))


@pytest.mark.parametrize("sort", SORTS)
def test_ensemble_instances_match_oracle_alone(sort):
    """Each instance of a batched ensemble evolves exactly as the oracle runs
    it alone: RNG keys, cells and slots are instance-local."""
    inst = []
    counts = [1200, 3000, 800, 2500]
    for k, n in enumerate(counts):
        side = float((n / 1500.0) ** (1 / 3))
        inst.append(dict(box_lo=(0.0, 0.0, 0.0), box_hi=(side, side, side), seed=100 + k,
                         d_scale=[0.5, 1.0, 2.0, 1.5][k], k2_scale=[1.0, 2.0, 0.5, 3.0][k]))
    s = System(dt=1e-3, seed=1, normals="table", instances=inst, sort=sort)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 3.0)
    u = s.add_reaction(1, [Cc], [A, B], 50.0)
    s.set_product_placement(u, L.BD_PP_UNBINDRAD, 0.01)
    s.add_reaction(0, [], [A], 500.0)
    s.finalize()
    g = rng(20)
    pos, sp = [], []
    for d, n in zip(inst, counts):
        pos.append(uniform_positions(g, n, d["box_lo"], d["box_hi"]))
        sp.append((np.arange(n) % 2).astype(np.int32))
    s.set_ensemble_particles(np.concatenate(pos), np.concatenate(sp), counts)
    oracles = [orc.OracleSystem(s, instance=k) for k in range(len(counts))]
    recs = [orc.records(p, q, inst=k) for k, (p, q) in enumerate(zip(pos, sp))]
    for t in range(15):
        s.step(1)
        s.synchronize()
        xyz, w = s.slots()
        got = orc.slots_to_records(xyz, w)
        for k, o in enumerate(oracles):
            recs[k] = o.step(t, recs[k])["recs"]
            live = recs[k][recs[k][:, 3] != 0xFFFFFFFF]
            mine = got[(got[:, 3] != 0xFFFFFFFF) & ((got[:, 3] >> 16) == k)]
            np.testing.assert_array_equal(mine, live, err_msg=f"instance {k} step {t}")
    np.testing.assert_array_equal(s.instance_counts(),
                                  [int(np.sum(r[:, 3] != 0xFFFFFFFF)) for r in recs])


def test_bin_overflow_grows_and_replays_exactly():
    """A cluster far denser than the planned occupancy overflows the cell
    bins: the bins grow, the step is replayed, and the result equals the
    oracle's and the compact sort's."""
    def make(sort):
        s = System((0, 0, 0), (2.0, 2.0, 2.0), dt=1e-3, seed=21, normals="table", sort=sort)
        A, B, Cc = s.add_species(0.2), s.add_species(0.2), s.add_species(0.1)
        s.add_reaction(2, [A, B], [Cc], 1.0)
        s.finalize()
        g = rng(21)
        pos = uniform_positions(g, 6000, (0, 0, 0), (2.0, 2.0, 2.0))
        pos[:600] = uniform_positions(g, 600, (0.9, 0.9, 0.9), (0.95, 0.95, 0.95))  # one cell's worth x 200
        s.set_particles(pos, (np.arange(6000) % 2).astype(np.int32))
        return s
    binned, compact = make("binned"), make("compact")
    _, npairs, ev = run_parity(binned, 6)
    assert npairs > 0 and ev[0] > 0
    compact.step(6)
    compact.synchronize()
    np.testing.assert_array_equal(gpu_records(binned), gpu_records(compact))
    assert np.diff(binned.cells()).max() > 100


@pytest.mark.parametrize("sort", SORTS)
def test_large_system_bit_exact(sort):
    """1.2M particles, species in contiguous blocks of the initial array: the
    streaming kernels' grid-stride loops wrap several times per thread and
    the pair kernel takes several cell tasks per warp, so a record read from
    the wrong chunk or a cell handled twice changes species counts and
    positions and shows here."""
    side = 31.0
    s = System((0, 0, 0), (side,) * 3, dt=1e-3, seed=26, normals="table", sort=sort)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.05)
    s.add_reaction(1, [Cc], [], 5.0)
    s.finalize()
    n = 1_200_000
    g = rng(26)
    pos = uniform_positions(g, n, (0, 0, 0), (side,) * 3)
    sp = np.repeat(np.arange(3, dtype=np.int32), [n // 2, n // 2 - n // 10, n // 10])
    s.set_particles(pos, sp)
    _, npairs, ev = run_parity(s, 3)
    assert npairs > 100 and ev[0] > 100


@pytest.mark.parametrize("sort", SORTS)
def test_clusters_across_cell_corners_bit_exact(sort):
    """Dense clusters around a cell corner make eight neighbouring cells
    large (more than 128 records: sorted by the large-cell kernels), next to
    ordinary cells: pairs inside large cells, between two large cells and
    between a large and an ordinary cell must all match the oracle."""
    side, n, n_cl = 2.0, 6000, 1600

    def make(pos, sp):
        s = System((0, 0, 0), (side,) * 3, dt=1e-3, seed=27, normals="table", sort=sort)
        A, B, Cc = s.add_species(0.2), s.add_species(0.2), s.add_species(0.1)
        s.add_reaction(2, [A, B], [Cc], 0.5)
        s.finalize()
        s.set_particles(pos, sp)
        return s
    g = rng(27)
    pos = uniform_positions(g, n, (0, 0, 0), (side,) * 3)
    sp = (np.arange(n) % 2).astype(np.int32)
    probe = make(pos, sp)
    dims, cell, _ = probe.grid()
    probe.close()
    corner = np.array([6, 6, 6], np.float32) * cell.astype(np.float32)
    pos[:n_cl] = uniform_positions(g, n_cl, corner - 0.04, corner + 0.04)
    c3 = np.clip(np.floor(pos / cell.astype(np.float32)).astype(np.int64), 0, dims.astype(np.int64) - 1)
    occupancy = np.bincount((c3[:, 2] * dims[1] + c3[:, 1]) * dims[0] + c3[:, 0])
    assert np.sum(occupancy > 128) >= 4  # large cells at the start
    s = make(pos, sp)
    _, npairs, ev = run_parity(s, 5)
    assert npairs > 0 and ev[0] > 0


@pytest.mark.parametrize("sort", SORTS)
def test_sparse_clumps_bit_exact(sort):
    """About a million small cells, most of them empty, with the particles in
    small clumps: the pair kernel's warps string many tasks (32 cells each)
    into one record stream, most tasks empty and the rest holding a few
    records, so rounds that the open tasks cannot fill, tasks opened after
    such a round and empty tasks between full ones all occur.  A record
    skipped or taken twice changes the slots and the pairs."""
    side, n_clumps, per = 20.0, 3000, 24
    s = System((0, 0, 0), (side,) * 3, dt=1e-3, seed=41, normals="table", sort=sort, cell_size=0.2)
    A, B, Cc = s.add_species(0.05), s.add_species(0.05), s.add_species(0.02)
    s.add_reaction(2, [A, B], [Cc], 0.2)
    s.finalize()
    g = rng(41)
    centres = uniform_positions(g, n_clumps, (0.2, 0.2, 0.2), (side - 0.2,) * 3)
    pos = np.repeat(centres, per, axis=0) + (g.random((n_clumps * per, 3), dtype=np.float32) - 0.5) * 0.3
    pos = np.clip(pos, 0.0, side).astype(np.float32)
    sp = (np.arange(len(pos)) % 2).astype(np.int32)
    s.set_particles(pos, sp)
    dims, _, _ = s.grid()
    assert int(np.prod(dims.astype(np.int64))) >= 900_000
    _, npairs, ev = run_parity(s, 3)
    assert npairs > 100 and ev[0] > 0


@pytest.mark.parametrize("sort", SORTS)
def test_many_cells_scan_in_chunks_bit_exact(sort):
    """9.3M cells: more than the cell scan's CTAs hold in shared memory at
    once (two CTAs per SM, 24,576 counts each), so each CTA's range goes
    through shared memory in several chunks, summed and then scanned again
    chunk by chunk; the cell starts must equal the oracle's."""
    side = 21.0
    s = System((0, 0, 0), (side,) * 3, dt=1e-3, seed=43, normals="table", sort=sort, cell_size=0.1)
    A, B, Cc = s.add_species(1.0), s.add_species(1.0), s.add_species(0.5)
    s.add_reaction(2, [A, B], [Cc], 0.05)  # binding radius well below the 0.1 um cells
    s.finalize()
    n = 120_000
    pos = uniform_positions(rng(43), n, (0, 0, 0), (side,) * 3)
    s.set_particles(pos, (np.arange(n) % 2).astype(np.int32))
    dims, _, _ = s.grid()
    assert int(np.prod(dims.astype(np.int64))) > 2 * 160 * 24576
    run_parity(s, 2)


def test_steps_ordered_on_a_caller_stream():
    """bd_step_async on another stream gives the same trajectory as bd_step."""
    torch = pytest.importorskip("torch")
    a = dense_a_b(1500, 1500, 1.5, seed=28, kon=5.0)
    b = dense_a_b(1500, 1500, 1.5, seed=28, kon=5.0)
    st = torch.cuda.Stream()
    for _ in range(3):
        a.step(4)
        b.step(4, stream=st.cuda_stream)
    st.synchronize()
    a.synchronize()
    b.synchronize()
    np.testing.assert_array_equal(gpu_records(a), gpu_records(b))


@pytest.mark.parametrize("sort", SORTS)
def test_competing_reactions_bit_exact(sort):
    """Three reactions of one pair compete (pair_mode CHANNELS): the chosen
    reaction of every accepted pair, its products and the event counters
    equal the oracle's."""
    s = System((0, 0, 0), (1.5, 1.5, 1.5), dt=1e-3, seed=29, normals="table", sort=sort, pairs="channels")
    A, B, Cc, D = (s.add_species(d) for d in (1.0, 1.0, 0.5, 0.3))
    s.add_reaction(2, [A, B], [Cc], 1.0)
    s.add_reaction(2, [B, A], [D], 0.5)
    r = s.add_reaction(2, [A, B], [Cc, D], 2.0)
    s.set_product_placement(r, L.BD_PP_UNBINDRAD, 0.02)
    s.add_reaction(2, [Cc, D], [A], 0.5)
    s.finalize()
    g = rng(29)
    pos = uniform_positions(g, 6000, (0, 0, 0), (1.5, 1.5, 1.5))
    s.set_particles(pos, (np.arange(6000) % 2).astype(np.int32))
    _, npairs, ev = run_parity(s, 15)
    assert ev[0] > 30 and ev[1] > 10 and ev[2] > 60


def test_handles_step_concurrently_as_alone():
    """Two handles stepping at the same time on their own streams, each
    with cooperative launches that fill the GPU (the cell scan over every
    SM, the matcher's grid on a dense system), give the results each gives
    alone: the launches of one handle never wait on CTAs of the other."""
    from gpusmoldyn_gb300 import configs

    def big(seed):
        side = 200.0 * (8_000_000 / 16_000_000) ** (1 / 3)
        return configs.build_c3(n=8_000_000, side=side, seed=seed, normals="table")

    def dense(seed):
        return dense_a_b(2000, 2000, 2.0, seed=seed, kon=5.0)

    alone = []
    for make, seed in ((big, 51), (dense, 52)):
        s = make(seed)
        s.step(20)
        s.synchronize()
        alone.append(gpu_records(s))
        s.close()
    a, b = big(51), dense(52)
    a.step(20)
    b.step(20)
    a.synchronize()
    b.synchronize()
    np.testing.assert_array_equal(gpu_records(a), alone[0])
    np.testing.assert_array_equal(gpu_records(b), alone[1])
