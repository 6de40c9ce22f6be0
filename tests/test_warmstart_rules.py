"""Host logic of the warm-start study (mf-lbm-cuda_gb300/mflbm/warmstart.py):
the two stopping rules read from a recorded permeability trajectory, and the
fallback to the cold start, on a scripted context (no GPU)."""
import pytest

from mflbm import warmstart


def test_band_steps_first_step_from_which_k_stays_in_band():
    traj = [(50, 0.5), (100, 0.995), (150, 1.02), (200, 1.009), (250, 0.999), (300, 1.0)]
    assert warmstart.band_steps(traj, 1.0, 0.01) == 200
    assert warmstart.band_steps(traj, 1.0, 0.05) == 100
    assert warmstart.band_steps(traj[:3], 1.0, 0.01) is None     # last point outside
    assert warmstart.band_steps([(50, 1.0)], 1.0, 0.01) == 50


class _Scripted:
    """Context whose k follows k_of(steps since the last start)."""

    def __init__(self, k_of):
        self.k_of, self.t, self.runs = k_of, 0, []

    def run(self, nt, n):
        self.runs.append((nt, n))
        self.t += n

    def restart(self):
        self.t = 0


@pytest.fixture
def scripted(monkeypatch):
    monkeypatch.setattr(warmstart, "permeability", lambda ctx, case: ctx.k_of(ctx.t))
    return _Scripted


def test_record_run_stops_at_the_convergence_rule(scripted):
    ctx = scripted(lambda t: 1.0 - 0.5 ** (t / 100.0))
    traj, fell, steps = warmstart.record_run(ctx, None, tol=1e-3, interval=500, max_steps=10000, every=50)
    assert fell is None and steps == traj[-1][0] and len(traj) == steps // 50
    k = dict(traj)
    assert abs(k[steps] - k[steps - 500]) <= 1e-3 * k[steps]
    assert abs(k[steps - 50] - k[steps - 550]) > 1e-3 * k[steps - 50]
    assert ctx.runs[0] == (1, 50) and ctx.runs[1] == (51, 50)    # step counters continue


def test_record_run_falls_back_and_restarts_the_window(scripted):
    ctx = scripted(lambda t: 2.0 if t < 10 ** 9 else 0.0)
    ctx.k_of = lambda t: 1.0 - 0.5 ** (t / 100.0)
    calls = []

    def fallback():
        calls.append(ctx.t)
        ctx.restart()
    traj, fell, steps = warmstart.record_run(ctx, None, 1e-3, 500, 10000, 50, check=lambda k: False,
                                             on_fallback=fallback)
    assert calls == [500] and fell == 500
    assert ctx.runs[10] == (1, 50)                               # counters restart with the cold start
    assert steps - fell >= 500
    # the record after the fallback is the cold start's from its own step 50
    assert dict(traj)[550] == pytest.approx(1.0 - 0.5 ** 0.5)


def test_predicted_permeability_sums_fluid_voxels_only():
    """The network's outputs at solid voxels are untrained (the loss masks
    them) and the fill sets them to rest: they must not enter the predicted
    permeability."""
    import numpy as np
    from mflbm import unet
    nx, ny, nz = 6, 4, 5
    walls = np.zeros((nz, ny, nx), np.int32)
    walls[:, :, 0] = walls[:, :, -1] = 1          # the x walls
    walls[2, 1, 3] = 1                             # one grain voxel
    y = np.zeros((nz, ny, nx, 4), np.float32)
    y[..., 2] = 0.5
    y[walls != 0, 2] = 1e6                         # garbage where the network is not trained
    scales = np.array([1, 1, 2, 1], np.float32)
    k = unet.predicted_permeability(y, scales, nx, ny, nz, walls)
    fluid = int((walls == 0).sum())
    assert k == pytest.approx(0.5 * 2 * fluid / ((nx - 2) * ny * nz))
