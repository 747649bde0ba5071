"""The MD serving loop (irr_serve_run): continuous batching, admission, isolation (GPU)."""
import pytest

pytestmark = pytest.mark.gpu

SMALL = dict(num_jobs=8, steps_per_job=25, rebuild_every=10, min_atoms=2048, max_atoms=12000,
             arrival_rate=2000.0, seed=12345)


def test_each_job_is_the_same_alone_and_in_the_mix(built_lib):
    import irregular_gb300 as irr
    stats, jobs = irr.serve(**SMALL)
    assert stats.jobs_done == SMALL["num_jobs"] and stats.rejected == 0
    assert stats.max_resident > 1, "jobs should overlap at this arrival rate"
    for k in (0, 3, 7):
        s1, alone = irr.serve(only_job=k, **SMALL)
        assert s1.jobs_done == 1
        assert alone[k].state_hash == jobs[k].state_hash
        assert alone[k].energy == jobs[k].energy
    _, serial = irr.serve(mode=irr.IRR_SERVE_SERIAL, **SMALL)
    assert [j.state_hash for j in serial] == [j.state_hash for j in jobs]


def test_budget_limits_residency(built_lib):
    import irregular_gb300 as irr
    # the largest job of this stream needs < 12000 * 1600 B + 64 MiB; allow two of them
    budget = 2 * (12000 * 1600 + (64 << 20)) + 1
    stats, jobs = irr.serve(budget_bytes=float(budget), **SMALL)
    assert stats.jobs_done == SMALL["num_jobs"]
    assert 1 <= stats.max_resident <= 2
    assert stats.peak_budget_bytes <= budget
    assert all(j.done_s >= j.admit_s >= j.arrival_s for j in jobs)


def test_job_larger_than_the_budget_is_rejected(built_lib):
    import irregular_gb300 as irr
    stats, jobs = irr.serve(budget_bytes=1e6, **SMALL)
    assert stats.rejected == SMALL["num_jobs"] and stats.jobs_done == 0
    assert all(j.status == irr.IRR_ERR_BUDGET for j in jobs)


def test_latency_statistics(built_lib):
    import irregular_gb300 as irr
    stats, jobs = irr.serve(**SMALL)
    assert 0 < stats.p50_ms <= stats.p99_ms <= stats.max_ms
    assert stats.edges_per_s > 0 and stats.pair_evals > 0
    lat = sorted(1e3 * (j.done_s - j.arrival_s) for j in jobs)
    assert abs(stats.max_ms - lat[-1]) < 1e-6


def test_shortest_job_first_admission(built_lib):
    """One slot, every job waiting from the start: SJF admits them smallest
    first (FIFO in arrival order), and each job's trajectory is the same."""
    import irregular_gb300 as irr
    cfg = dict(SMALL, arrival_rate=1e9, max_resident=1)
    _, fifo = irr.serve(**cfg)
    _, sjf = irr.serve(policy=irr.IRR_SERVE_SJF, **cfg)
    by_admit = sorted(range(len(sjf)), key=lambda k: sjf[k].admit_s)
    atoms = [sjf[k].atoms for k in by_admit]
    assert atoms[1:] == sorted(atoms[1:])  # the first admission may precede the last arrival
    assert [j.state_hash for j in sjf] == [j.state_hash for j in fifo]


def test_serial_plain_schedule(built_lib):
    """IRR_SERVE_SERIAL_PLAIN: one job at a time, every force by the plain
    edge-parallel kernel (atomics: another summation order, so the final
    energies agree with the partitioned schedule's to FP32 reordering, not
    bit for bit)."""
    import irregular_gb300 as irr
    stats, plain = irr.serve(mode=irr.IRR_SERVE_SERIAL_PLAIN, **SMALL)
    assert stats.jobs_done == SMALL["num_jobs"] and stats.max_resident == 1
    _, serial = irr.serve(mode=irr.IRR_SERVE_SERIAL, **SMALL)
    for p, s in zip(plain, serial):
        assert p.status == 0 and p.edges == s.edges
        assert abs(p.energy - s.energy) <= 1e-5 * abs(s.energy)
