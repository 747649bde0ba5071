"""The serving stream's jobs as the host makes them (irr_serve_job_state; CPU, no GPU)."""
import numpy as np


def test_job_state_is_deterministic_fcc(built_lib):
    import irregular_gb300 as irr
    cfg = dict(num_jobs=6, seed=777, min_atoms=2048, max_atoms=40000)
    sizes = irr.serve_job_sizes(**cfg)
    assert len(sizes) == 6
    for k, n in enumerate(sizes):
        cells = round((n / 4) ** (1 / 3))
        assert n == 4 * cells ** 3 and n >= 2048
        atoms, side, pos, vel = irr.serve_job_state(k, **cfg)
        assert atoms == n and pos.shape == (n, 3) and vel.shape == (n, 3)
        assert np.all(pos >= 0) and np.all(pos < side)
        assert abs(side - cells * (4 / 0.8442) ** (1 / 3)) < 1e-12 * side
        # Maxwell velocities: zero momentum, kinetic temperature 1.44 exactly
        assert np.abs(vel.sum(axis=0)).max() < 1e-9 * n
        assert abs((vel * vel).sum() / (3 * n - 3) - 1.44) < 1e-12
        again = irr.serve_job_state(k, **cfg)
        assert np.array_equal(again[2], pos) and np.array_equal(again[3], vel)
    # another seed gives other jobs
    assert irr.serve_job_sizes(num_jobs=6, seed=778, min_atoms=2048, max_atoms=40000) != sizes


def test_job_state_rejects_bad_arguments(built_lib):
    import irregular_gb300 as irr
    import pytest
    with pytest.raises(irr.IrregularError):
        irr.serve_job_state(6, num_jobs=6)
    with pytest.raises(irr.IrregularError):
        irr.serve_job_state(-1, num_jobs=6)


def test_state_digest_is_order_and_bit_sensitive(built_lib):
    import irregular_gb300 as irr
    rng = np.random.default_rng(1)
    x = rng.random((100, 3))
    d = irr.state_digest(x)
    assert d == irr.state_digest(x.copy())
    y = x.copy()
    y[5, 1] = np.nextafter(y[5, 1], 2.0)
    assert irr.state_digest(y) != d
    assert irr.state_digest(x[::-1]) != d
