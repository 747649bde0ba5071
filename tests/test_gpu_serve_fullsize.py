"""The served stream at its full job sizes (GPU): Poisson arrivals at 200 jobs/s,
each an LJ system of log-uniform size in [2,048, 2,097,152] atoms at density
0.8442 asking for 50 velocity-Verlet steps, under a 120 GB admission budget.

A stream of 16 jobs that holds at least one job of more than 1,048,576 atoms
runs with continuous batching.  Its largest job is then checked two ways:
  * bit for bit: the same initial state (irr_serve_job_state) run alone
    through irr_md reaches the state digest the job reported from the mix;
  * against FP64: the oracle MD run on that job alone, its FP64 forces
    evaluated at the float copy of the positions as the GPU's FP32 reduction
    does (so that only the per-edge arithmetic differs), ends at the same total
    energy to 1e-7, and within 1e-5 in positions and 1e-4 in velocities at the
    99th percentile of atoms (1e-4 and 1e-2 at the worst): each step a few
    atoms' float copies round an ulp apart in the two runs, and the gap spreads
    from them.
"""
import numpy as np
import pytest

from helpers import trajectory_gap

pytestmark = pytest.mark.gpu

BIG = 1048576


def stream_config(irr):
    """The default stream (200 jobs/s, 2,048 to 2,097,152 atoms, 50 steps, 120 GB),
    16 jobs, at the first seed from 20260005 on whose jobs include one above
    BIG atoms (the sizes are made on the host, no GPU)."""
    for seed in range(20260005, 20260005 + 64):
        cfg = dict(num_jobs=16, seed=seed)
        sizes = irr.serve_job_sizes(**cfg)
        if max(sizes) > BIG:
            return cfg, sizes
    raise AssertionError("no seed with a job above 1,048,576 atoms")


def test_largest_job_of_a_mixed_stream(built_lib, oracle_lib):
    import irregular_gb300 as irr
    O = oracle_lib
    cfg, sizes = stream_config(irr)
    stats, jobs = irr.serve(**cfg)
    assert stats.jobs_done == cfg["num_jobs"] and stats.rejected == 0
    assert stats.max_resident > 1
    big = int(np.argmax(sizes))
    assert jobs[big].atoms == sizes[big] > BIG and jobs[big].status == 0

    atoms, side, pos, vel = irr.serve_job_state(big, **cfg)
    assert atoms == sizes[big]
    md = irr.MD(pos, vel, side, dt=0.005, cutforce=2.5, skin=0.3, rebuild_every=20)
    md.run(50)
    gp, gv = md.state()
    ke, pe, _ = md.energy()
    md.close()
    assert irr.state_digest(gp) == jobs[big].state_hash
    assert abs((ke + pe) - jobs[big].energy) <= 1e-12 * abs(jobs[big].energy)

    rp, rv, rke, rpe = O.md_run(pos, vel, side, 2.5, 0.3, 0.005, 50, 20, float_forces=True)
    gap = trajectory_gap(gp, gv, rp, rv, side)
    assert gap["dx_p99"] <= 1e-5 and gap["dv_p99"] <= 1e-4, gap
    assert gap["dx_max"] <= 1e-4 and gap["dv_max"] <= 1e-2, gap
    assert abs((ke + pe) - (rke + rpe)) <= 1e-7 * abs(rke + rpe)
