"""The GPU MD loop (irr_md_*) against the FP64 reference MD of the oracle (GPU)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def system(cells=6, rho=0.8442, temp=1.44, seed=20260003, jitter=0.03):
    import workloads as W
    pos, side = W.fcc_lattice(cells, cells, cells, rho)
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = (pos + rng.normal(0, jitter, pos.shape)) % side
    vel = W.maxwell_velocities(pos.shape[0], temp, seed + 1)
    return pos, vel, side


@pytest.mark.parametrize("cells", [4, 6, 12])
def test_initial_forces_match_fp64(built_lib, oracle_lib, cells):
    """cells 4: two list cells per axis (the half list, then the partition's
    node order and row layout); 6 and 12: 3 and 7 cells per axis (atoms sorted
    by cell, rows written in order by the cell search; at 7 cells each pair's
    image is decided by its cell)."""
    import irregular_gb300 as irr
    O = oracle_lib
    pos, vel, side = system(cells=cells)
    md = irr.MD(pos, vel, side)
    f = md.forces()
    # FP64 forces of the positions the GPU computes with (the float copy of
    # the FP64 state), list at 2.8
    p32 = pos.astype(np.float32)
    edges = O.neighbor_half_list(p32, float(np.float32(side)), np.float32(2.8 ** 2))
    f64, sabs = O.lj_reduce_f64(p32.astype(np.float64), edges, O.lj_param(2.5 ** 2, side, True))
    f64 *= 48.0
    assert np.abs(f - f64).max() / np.abs(f64).max() <= 1e-6
    assert md.info().num_edges == edges.shape[0]
    md.close()


@pytest.mark.parametrize("cells,reorder_every", [(4, 1), (4, 10), (6, 10), (12, 10)])
def test_short_trajectory_matches_fp64_reference(built_lib, oracle_lib, cells, reorder_every):
    """cells 4 (two list cells per axis): reorder_every 1 re-sorts the atoms
    at the second rebuild, 10 keeps their order; cells 6 and 12 re-sort by
    cell at every rebuild (either way the same physics)."""
    import irregular_gb300 as irr
    O = oracle_lib
    pos, vel, side = system(cells=cells)
    steps = 25  # crosses one rebuild (every 20 steps)
    md = irr.MD(pos, vel, side, dt=0.005, rebuild_every=20, reorder_every=reorder_every)
    md.run(steps)
    gp, gv = md.state()
    info = md.info()
    assert info.steps == steps and info.rebuilds == 2  # the initial build + one
    rp, rv, _, _ = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, steps, 20)
    dx = gp - rp
    dx -= side * np.round(dx / side)
    assert np.abs(dx).max() <= 1e-5
    assert np.abs(gv - rv).max() <= 1e-4
    md.close()


@pytest.mark.parametrize("cells", [4, 12])
def test_plain_force_path_matches_fp64(built_lib, oracle_lib, cells):
    """exec_plain: the forces by the plain edge-parallel kernel over the half
    list taken from the rows (atomics), the same bound against FP64 and the
    same short trajectory as the reference MD."""
    import irregular_gb300 as irr
    O = oracle_lib
    pos, vel, side = system(cells=cells)
    md = irr.MD(pos, vel, side, exec_plain=True)
    f = md.forces()
    p32 = pos.astype(np.float32)
    edges = O.neighbor_half_list(p32, float(np.float32(side)), np.float32(2.8 ** 2))
    f64, _ = O.lj_reduce_f64(p32.astype(np.float64), edges, O.lj_param(2.5 ** 2, side, True))
    f64 *= 48.0
    assert np.abs(f - f64).max() / np.abs(f64).max() <= 1e-6
    assert md.info().num_edges == edges.shape[0]
    md.close()
    md = irr.MD(pos, vel, side, dt=0.005, rebuild_every=20, exec_plain=True)
    md.run(25)
    gp, gv = md.state()
    rp, rv, _, _ = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, 25, 20)
    dx = gp - rp
    dx -= side * np.round(dx / side)
    assert np.abs(dx).max() <= 1e-5
    assert np.abs(gv - rv).max() <= 1e-4
    md.close()


def test_neighbour_slots_overflow_gives_the_same_trajectory(built_lib):
    """row_slots = 8 (rows hold ~78): every rebuild's one-pass search
    overflows its slots and falls back to counting and writing in place; the
    rows, and so the trajectory, are bitwise those of the automatic slots."""
    import irregular_gb300 as irr
    pos, vel, side = system(cells=12)
    states = []
    for slots in (0, 8):
        md = irr.MD(pos, vel, side, dt=0.005, rebuild_every=10, row_slots=slots)
        md.run(45)  # the first build and four rebuilds
        assert md.info().rebuilds == 5
        states.append(md.state())
        md.close()
    for a, b in zip(states[0], states[1]):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_dilute_gas_takes_the_half_list_path(built_lib, oracle_lib):
    """A gas at density 0.03: 16 cells per axis but more cells than atoms, so
    the rebuild takes the half-stencil pair list and the partition instead of
    rows written in cell order; the list and the forces (per atom, against the
    sum of its terms' magnitudes) match the FP64 oracle, before and after a
    rebuild."""
    import irregular_gb300 as irr
    from helpers import TOL_PERNODE_F64, scaled_error
    O = oracle_lib
    # a simple cubic lattice (spacing 3.22 > the 2.8 list cutoff) with a 0.35
    # jitter: ~2,000 pairs inside 2.8, none closer than ~1.1
    a, m = (1 / 0.03) ** (1 / 3), 16
    side = float(np.float32(m * a))
    grid = np.stack(np.meshgrid(*(np.arange(m),) * 3, indexing="ij"), -1).reshape(-1, 3) * a
    rng = np.random.Generator(np.random.PCG64(41))
    pos = (grid + rng.normal(0, 0.35, grid.shape)) % side
    n = pos.shape[0]
    assert int(side / 2.8) ** 3 > n
    vel = rng.normal(0, 0.5, (n, 3))
    md = irr.MD(pos, vel, side, dt=0.002, rebuild_every=5)
    try:
        for steps in (0, 10):  # the initial build, then right after the second rebuild
            if steps:
                md.run(steps)
            pos, _ = md.state()
            q32 = pos.astype(np.float32)
            edges = O.neighbor_half_list(q32, float(np.float32(side)), np.float32(2.8 ** 2))
            assert md.info().num_edges == edges.shape[0] > 0
            f64, sabs = O.lj_reduce_f64(q32.astype(np.float64), edges, O.lj_param(2.5 ** 2, side, True))
            assert scaled_error(md.forces(), 48.0 * f64, 48.0 * sabs) <= TOL_PERNODE_F64
    finally:
        md.close()


def test_energy_and_momentum_conservation(built_lib):
    import irregular_gb300 as irr
    pos, vel, side = system(cells=8)
    md = irr.MD(pos, vel, side, dt=0.005)
    ke0, pe0, _ = md.energy()
    e0 = ke0 + pe0
    md.run(400)
    ke1, pe1, vir = md.energy()
    e1 = ke1 + pe1
    n = pos.shape[0]
    assert abs(e1 - e0) / abs(e0) <= 2e-3, (e0, e1)
    _, v = md.state()
    assert np.abs(v.sum(axis=0)).max() <= 1e-6 * n
    assert md.info().rebuilds == 1 + 400 // 20
    # temperature stays in the liquid's range
    t = 2.0 * ke1 / (3 * n - 3)
    assert 0.5 < t < 2.5
    md.close()


def test_energies_match_fp64(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    pos, vel, side = system()
    md = irr.MD(pos, vel, side)
    ke, pe, _ = md.energy()
    _, _, rke, rpe = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, 0, 20)
    assert abs(ke - rke) <= 1e-9 * abs(rke)
    assert abs(pe - rpe) <= 1e-5 * abs(rpe)
    md.close()


def test_bad_md_config_is_rejected(built_lib):
    import irregular_gb300 as irr
    pos, vel, side = system(cells=2)  # side 6.7 < 2 * (2.5 + 0.3)
    with pytest.raises(irr.IrregularError) as ei:
        irr.MD(pos, vel, side)
    assert ei.value.status == irr.IRR_ERR_ARG
