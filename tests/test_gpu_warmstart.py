"""What the trained network gains over the method without it: a U-Net
trained on the GPU by the library's own kernels, on converged flows of 128
seeded 64^3 packs, evaluated on held-out packs.

  * Its predicted flow field is closer to the converged field than the cold
    start's rest state (relative L2 error of u_z over the fluid nodes: the
    rest state's is 1 by definition) and closer than the untrained network's.
  * In time: 200 steps after the start, the flow started from the
    prediction is closer to the converged flow than the flow started from
    rest (the network saves the start-up transient).
  * The warm start converges to the same permeability as the cold start
    (within 0.1 %): starting from the prediction does not bias the answer.

The study in mflbm/warmstart.py measures the time to the 1e-5 convergence
criterion; there the gain is bounded by the oracle start (the fill from the
converged field itself), because the criterion's tail is set by a slow decay
that the fill does not remove."""
import numpy as np
import pytest

from mflbm import abi, lib, unet, warmstart

pytestmark = pytest.mark.gpu


def _uz_err(pred_raw, target, mask):
    m = mask > 0
    return float(np.linalg.norm((pred_raw[..., 2] - target[..., 2])[m]) / np.linalg.norm(target[..., 2][m]))


def test_trained_network_beats_the_rest_state(mflbm_lib):
    n = 64
    train = warmstart.sample_cases(128, n, 7000)
    data, _ = warmstart.generate(train, tol=1e-5, interval=500, max_steps=40000, log=lambda s: None)
    scales = warmstart.scales_of(data)
    held = warmstart.sample_cases(3, n, 9000)
    hdata, _ = warmstart.generate(held, tol=1e-5, interval=500, max_steps=40000, log=lambda s: None)
    net = unet.UNet(n, n, n, seed=5)
    untrained = [_uz_err(net.forward(x) * scales, t, m) for x, t, m in hdata]
    losses, _ = unet.train(net, [(x, t / scales, m) for x, t, m in data], epochs=40, lr=2e-3)
    assert losses[-1] < 0.85 * losses[1]
    trained = [_uz_err(net.forward(x) * scales, t, m) for x, t, m in hdata]
    assert np.mean(trained) < 0.9 and max(trained) < 1.0, trained
    assert np.mean(trained) < np.mean(untrained), (trained, untrained)
    ws = warmstart.WarmStarter(net.get_params(), scales)
    net.close()
    case = held[0]
    nu, g = warmstart.nu_g(case)
    cold, info = lib.setup_case(case, abi.MFLBM_FP32)
    k_cold, _, _ = warmstart.run_until_converged(cold, case, 1e-5, 500, 40000)
    cold.close()
    warm, info = lib.setup_case(case, abi.MFLBM_FP32)
    walls = info["walls_global"]
    pred = ws.predict(case, walls)
    unet.fill_from_prediction(warm, pred, walls, nu, g, ws.scales)
    k_warm, _, _ = warmstart.run_until_converged(warm, case, 1e-5, 500, 40000)
    warm.close()
    # the start-up transient: u_z error against the converged flow after 200 steps
    target, mask = hdata[0][1], hdata[0][2]
    errs = {}
    for how in ("cold", "warm"):
        c, _ = lib.setup_case(case, abi.MFLBM_FP32)
        if how == "warm":
            unet.fill_from_prediction(c, pred, walls, nu, g, ws.scales)
        c.run(1, 200)
        t, _ = unet.flow_target(c, walls, nu, g)
        errs[how] = _uz_err(t, target, mask)
        c.close()
    ws.close()
    assert errs["warm"] < errs["cold"], errs
    assert abs(k_warm - k_cold) <= 1e-3 * k_cold, (k_warm, k_cold)
