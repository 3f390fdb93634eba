"""The learned far-field surrogate.

CPU: the numpy restatement (oracle/surrogate_net.py) against finite differences.
GPU, through the C ABI:
  * the fused tensor-core forward kernel and the training forward pass against
    the restatement (BF16 inputs, parameters and hidden activations on both
    sides): 2e-3 of the largest output;
  * the training gradient against the restatement's: 1e-3 of its norm;
  * an ensemble trained on part of a full-sky shell's far keys: its Fisher
    matrix against the plain cubature's and against the method without the
    network (zero networks: every far key set to the point value xi_t(d)),
    and the ensemble-disagreement fallback.
"""
import numpy as np
import pytest

import surrogate_net as SO
from opsec_gpu import api, synth

PK = synth.pk_table()


def features(n, rng):
    """Inputs in the ranges the surrogate sees: d/1000, mu, 6 extents/100, k edges x 5, sin, cos."""
    f = np.zeros((n, 16))
    d = rng.uniform(50, 2000, n)
    f[:, 0] = d / 1000
    f[:, 1] = rng.uniform(0, 1, n)
    f[:, 2:8] = rng.uniform(0.05, 2.0, (n, 6))
    k = rng.uniform(0, 0.4, n)
    f[:, 8] = 5 * k
    f[:, 9] = 5 * (k + 0.01)
    f[:, 10] = np.sin((k + 0.005) * d)
    f[:, 11] = np.cos((k + 0.005) * d)
    return f


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = SO.init(3).astype(np.float64)
    p[SO.OFF["b1"]:SO.OFF["b1"] + 128] = rng.normal(0, 0.1, 128)
    x = features(40, rng)
    y = rng.normal(0, 0.3, 40)
    _, g = SO.loss_and_grad(p, x, y, rounded=False)
    idx = [rng.choice(np.arange(o, o + 128), 5, replace=False) for n, o in SO.OFF.items() if n != "b4"]
    for i in np.concatenate(idx + [[SO.OFF["b4"]]]):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (SO.loss(pp, x, y, rounded=False) - SO.loss(pm, x, y, rounded=False)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])


@pytest.mark.gpu
def test_surrogate_forward_and_gradient_against_restatement():
    rng = np.random.default_rng(2)
    sv, _ = synth.shell_survey(3, 4, 8)
    e = api.Engine(api.make_config(sv, bands=synth.band_edges(2, 0.0, 0.1)))
    p = SO.init(5)
    p[SO.OFF["b1"]:SO.OFF["b1"] + 128] = rng.normal(0, 0.1, 128)
    p[SO.OFF["b2"]:SO.OFF["b2"] + 128] = rng.normal(0, 0.1, 128)
    n = 300
    x = features(n, rng)
    y = rng.normal(0, 0.3, n)
    r = e.surrogate_eval(p, x, y)
    ref_out, _ = SO.forward(p.astype(np.float64), x)
    scale = np.max(np.abs(ref_out))
    print("max |out - ref| / max|ref|: simt", np.max(np.abs(r["out_simt"] - ref_out)) / scale,
          "tc", np.max(np.abs(r["out_tc"] - ref_out)) / scale)
    assert np.max(np.abs(r["out_simt"] - ref_out)) <= 2e-3 * scale
    assert np.max(np.abs(r["out_tc"] - ref_out)) <= 2e-3 * scale
    assert np.max(np.abs(r["out_tc"] - r["out_simt"])) <= 2e-3 * scale
    ref_loss, ref_g = SO.loss_and_grad(p.astype(np.float64), x, y.astype(np.float32).astype(np.float64))
    print("loss", r["loss"], ref_loss, "grad rel", np.linalg.norm(r["grad"] - ref_g) / np.linalg.norm(ref_g))
    assert abs(r["loss"] - ref_loss) <= 1e-3 * ref_loss
    assert np.linalg.norm(r["grad"] - ref_g) <= 1e-3 * np.linalg.norm(ref_g)
    sizes = {"W1": 2048, "b1": 128, "W2": 16384, "b2": 128, "W3": 16384, "b3": 128, "w4": 128, "b4": 1}
    for name, off in SO.OFF.items():  # every parameter block, not only the norm
        blk = slice(off, off + sizes[name])
        assert np.linalg.norm(r["grad"][blk] - ref_g[blk]) <= 5e-3 * np.linalg.norm(ref_g[blk]) + 1e-12, name
    e.close()


def fisher(sv, cells, counts, bands, M, extra, weights=None):
    e = api.Engine(api.make_config(sv, bands=bands, extra=extra))
    e.set_pk(*PK)
    if weights is not None:
        e.surrogate_weights(weights)
    r = e.fisher_build(cells, counts, M)
    stats = e.surrogate_stats() if weights is not None else None
    e.close()
    return r, stats


@pytest.mark.gpu
def test_surrogate_gain_and_fallback():
    """An ensemble trained on half of a shell's far (key, table) samples, applied
    to all of its far keys.  Accepting every prediction must beat the method
    without the network (zero networks: the point value xi_t(d) for every far
    key) by 5x in the Fisher matrix.  The members' disagreement is the guard:
    as its tolerance tightens, fewer far keys are predicted and the Fisher error
    falls, down to the plain build when none is.  Measured on this 8 x 12 x 24
    shell: tol 0.1 predicts 97 % of the far keys at 4.5e-2, tol 0.05 22 % at
    6.9e-3, tol 0.02 none; no tolerance reaches the 1e-3 target with keys
    predicted (the learned form's target is not met, and this test says so)."""
    bands = synth.band_edges(20, 0.0, 0.2)
    sv, cells = synth.shell_survey(8, 12, 24)
    counts = synth.grf_counts(sv, cells)
    M = 400
    et = api.Engine(api.make_config(sv, bands=bands))
    et.set_pk(*PK)
    info = et.surrogate_train(max_samples=276_000, epochs=30, seed=1)
    w = et.surrogate_weights()
    et.close()
    plain, _ = fisher(sv, cells, counts, bands, M, [])
    all_in, st = fisher(sv, cells, counts, bands, M, ["surrogate = 1", "surrogate.tol = 1e9"], w)
    zero = np.zeros_like(w)
    zero[-1] = w[-1]
    point, st0 = fisher(sv, cells, counts, bands, M, ["surrogate = 1", "surrogate.tol = 1e9"], zero)
    sc = np.max(np.abs(plain["F"]))
    err = {name: np.max(np.abs(r["F"] - plain["F"])) / sc for name, r in (("network", all_in), ("point value", point))}
    print("training:", info)
    print(f"far keys {st['far']}; " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    assert st["predicted"] == st["far"] and st0["predicted"] == st0["far"]
    assert err["network"] < 0.2 * err["point value"], err
    guarded = {}
    for tol in (0.1, 0.05, 0.02, 0.01, 0.005):
        r, stg = fisher(sv, cells, counts, bands, M, ["surrogate = 1", f"surrogate.tol = {tol}"], w)
        guarded[tol] = (stg["predicted"] / st["far"], float(np.max(np.abs(r["F"] - plain["F"])) / sc))
    print("tol: (fraction of far keys predicted, Fisher rel err)", guarded)
    fr = [guarded[t][0] for t in sorted(guarded, reverse=True)]
    er = [guarded[t][1] for t in sorted(guarded, reverse=True)]
    assert all(a >= b for a, b in zip(fr, fr[1:])), guarded        # coverage falls with the tolerance
    assert all(a >= b - 1e-12 for a, b in zip(er, er[1:])), guarded  # and so does the error
    assert fr[0] > 0.9 and er[-1] <= 1e-12, guarded                  # from nearly all keys to none
