"""The miniMD-style MD workload at full size (GPU): FCC 4 x 64^3 = 1,048,576
atoms at reduced density 0.8442, Maxwell velocities at T = 1.44, cutoff 2.5,
skin 0.3, neighbour rebuild every 20 steps, velocity Verlet with dt = 0.005.

The FP64 oracle MD is too slow for the whole run at this size, so the check is
split into what it can do here and what does not depend on size:
  * the forces of a seeded sample of 2,000 atoms against FP64 (the law on the
    float positions the GPU computes with) at step 0 -- the perfect lattice,
    where every force cancels to ~0 by symmetry, so the error is bounded per
    node by the sum of its terms' magnitudes -- and right after the first
    neighbour rebuild (step 20), normwise and per result;
  * the whole system's trajectory against the FP64 oracle MD: after 5 steps
    with the oracle's forces evaluated on the FP64 positions (the GPU evaluates
    them on their float32 copy, whose rounding at this box side, ulp(107) =
    7.6e-6, moves the forces by ~1e-3 and the velocities by ~1e-5), and after 5,
    20 and 220 steps with the oracle evaluating its FP64 forces at the same
    float copy, which leaves only the FP32 per-edge arithmetic between them.
    The float copy is a step function of the FP64 position: each step a few
    of the atoms whose positions differ by ~1e-10 round their copies an ulp
    apart, and those atoms' neighbours feel it, so the per-atom gap grows from
    ~1e-9 (99th percentile after 5 steps) to ~1e-7 after 20; the bounds are
    per quantile, and the total energy is the sharp check;
  * over steps 20 to 220 the total momentum stays zero to rounding, and the
    total energy changes as the FP64 oracle's does (the melting lattice's
    energy exchange makes both drift by ~1e-3).
"""
import numpy as np
import pytest

from helpers import (TOL_PERNODE_F64, TOL_RESULT_MAX, TOL_RESULT_P50, result_error_summary,
                     scaled_error, trajectory_gap)

pytestmark = pytest.mark.gpu

CELLS = 64
RHO = 0.8442
TEMP = 1.44
SEED = 20260003
SAMPLE = 2000


def sample_forces_fp64(irr, O, pos64, side, sample):
    """FP64 forces (x48: the MD's force units), the per-component sum of the
    terms' magnitudes and the per-result scale of the sampled atoms, from every
    pair within the list radius that touches them."""
    p32 = pos64.astype(np.float32)
    d_edges = irr.neighbor_build(p32, float(np.float32(side)), 2.8 ** 2)
    edges = d_edges.to_host()
    d_edges.close()
    sel = np.zeros(p32.shape[0], bool)
    sel[sample] = True
    inc = edges[sel[edges[:, 0]] | sel[edges[:, 1]]]
    p = O.lj_param(2.5 ** 2, side, True)
    f64, sabs = O.lj_reduce_f64(p32.astype(np.float64), inc, p)
    sinf = O.lj_edge_scale_inf(p32.astype(np.float64), inc, p)
    return 48.0 * f64[sample], 48.0 * sabs[sample], 48.0 * sinf[sample]


@pytest.fixture(scope="module")
def system(built_lib, oracle_lib):
    import irregular_gb300 as irr
    import workloads as W
    pos, side = W.fcc_lattice(CELLS, CELLS, CELLS, RHO)
    vel = W.maxwell_velocities(pos.shape[0], TEMP, SEED)
    rng = np.random.Generator(np.random.PCG64(SEED + 7))
    sample = np.sort(rng.choice(pos.shape[0], SAMPLE, replace=False))
    return dict(irr=irr, O=oracle_lib, pos=pos, vel=vel, side=side, sample=sample)


def test_full_size_md(system):
    irr, O = system["irr"], system["O"]
    pos, vel, side, sample = system["pos"], system["vel"], system["side"], system["sample"]
    n = pos.shape[0]
    assert n == 1048576
    md = irr.MD(pos, vel, side, dt=0.005, cutforce=2.5, skin=0.3, rebuild_every=20)

    # step 0, the perfect lattice: forces cancel, the error is bounded per node
    f = md.forces()[sample]
    g, sabs, _ = sample_forces_fp64(irr, O, pos, side, sample)
    assert np.abs(g).max() < 1e-3 * sabs.max()  # ~0 by symmetry
    assert scaled_error(f, g, sabs) <= TOL_PERNODE_F64

    def close(gp, gv, rp, rv, bounds):
        gap = trajectory_gap(gp, gv, rp, rv, side)
        assert all(gap[k] <= b for k, b in bounds.items()), gap

    # the first 5 steps of the whole system against the FP64 oracle MD
    md.run(5)
    gp, gv = md.state()
    rp, rv, _, _ = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, 5, 20)
    close(gp, gv, rp, rv, {"dx_max": 1e-6, "dv_max": 1e-4})
    fp, fv, _, _ = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, 5, 20, float_forces=True)
    close(gp, gv, fp, fv, {"dx_p99": 1e-9, "dx_max": 1e-6, "dv_p99": 1e-7, "dv_max": 1e-4})

    # right after the first rebuild (step 20): forces of the current positions
    md.run(15)
    info = md.info()
    assert info.steps == 20 and info.rebuilds == 2
    gp, gv = md.state()
    # (from step 0 again: the oracle rebuilds its list at its first step and
    # every 20th after, so only an unbroken run keeps the GPU's schedule, and
    # a list of another age lacks other near-cutoff pairs of fast atoms)
    fp, fv, fke0, fpe0 = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, 20, 20, float_forces=True)
    close(gp, gv, fp, fv, {"dx_p99": 1e-6, "dx_max": 1e-4, "dv_p99": 1e-4, "dv_max": 1e-2})
    f = md.forces()[sample]
    g, sabs, sinf = sample_forces_fp64(irr, O, gp, side, sample)
    assert np.abs(f - g).max() / np.abs(g).max() <= 1e-6
    assert scaled_error(f, g, sabs) <= TOL_PERNODE_F64
    err = result_error_summary(f, g, sinf)
    assert err["p50"] <= TOL_RESULT_P50 and err["max"] <= TOL_RESULT_MAX, err

    # 200 more steps: momentum stays zero to rounding; the energy follows FP64's
    ke0, pe0, _ = md.energy()
    assert abs((ke0 + pe0) - (fke0 + fpe0)) <= 1e-7 * abs(fke0 + fpe0)
    md.run(200)
    ke1, pe1, _ = md.energy()
    _, v = md.state()
    vrms = np.sqrt((v * v).sum() / n)
    assert np.abs(v.sum(axis=0)).max() <= 1e-7 * n * vrms
    _, _, fke1, fpe1 = O.md_run(fp, fv, side, 2.5, 0.3, 0.005, 200, 20, float_forces=True)
    e0, e1, f1 = ke0 + pe0, ke1 + pe1, fke1 + fpe1
    assert abs(e1 - f1) <= 1e-6 * abs(f1), (e1, f1)
    drift = abs(e1 - e0) / abs(e0)
    assert drift <= 3e-3, drift
    assert md.info().rebuilds == 12
    md.close()
