"""Learned guide: the GPU network (BF16 tensor-core MLP, FP32 accumulation)
against the torch FP64 oracle (oracle/nn_oracle.py) for the forward pass
and the training gradient, and the guided render against plain PT."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LO, HI = [0.0, 0.0, 0.0], [10.0, 4.0, 10.0]


def random_inputs(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(LO, HI, (n, 3))
    nrm = rng.normal(size=(n, 3)); nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3)); wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    return np.hstack([pos, nrm, wo]).astype(np.float32)


def random_weights(seed):
    rng = np.random.default_rng(seed)
    w = []
    for l, (i, o) in enumerate([(64, 64), (64, 64), (64, 64), (64, 48)]):
        w.append(rng.normal(0, 0.5 if l == 3 else np.sqrt(2 / 64), i * o))
    return np.concatenate(w).astype(np.float32)


@pytest.mark.parametrize("encoding", [0, 1], ids=["freq", "oneblob"])
def test_forward_matches_oracle(gpu_lib, encoding):
    from cpppt import lib
    from oracle import nn_oracle
    w = random_weights(1)
    x = random_inputs(1000, 2)
    got = lib.nn_forward(w, LO, HI, x, encoding=encoding)
    ref = nn_oracle.forward(w, LO, HI, x, encoding=encoding)
    # mixture weights, selection probability and lobe means; bf16 activations
    assert np.abs(got[:, 40] - ref[:, 40]).max() < 2e-2
    wcols = [5 * j + 4 for j in range(8)]
    assert np.abs(got[:, wcols] - ref[:, wcols]).max() < 3e-2
    mcols = [5 * j + k for j in range(8) for k in range(3)]
    assert np.abs(got[:, mcols] - ref[:, mcols]).mean() < 1e-2
    kcols = [5 * j + 3 for j in range(8)]
    np.testing.assert_allclose(got[:, kcols], ref[:, kcols], rtol=5e-2, atol=2e-2)
    # the mixture weights sum to one
    np.testing.assert_allclose(got[:, wcols].sum(1), 1.0, atol=1e-5)


def _grad_records(n, seed):
    rng = np.random.default_rng(seed)
    x = random_inputs(n, seed + 2)
    wi = rng.normal(size=(n, 3)); wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    rec = np.zeros((n, 16), np.float32)
    rec[:, 0:9] = x
    rec[:, 9:12] = wi
    rec[:, 12] = rng.uniform(0.05, 0.5, n)
    rec[:, 13] = rng.exponential(1.0, n)
    return rec


# Per-layer agreement of the GPU weight gradient with the FP64 oracle.  The
# GPU keeps activations and the gradients of each layer's output in BF16
# (8-bit mantissa, relative rounding 2^-9) and sums the products over the
# batch in FP32; the oracle rounds the activations the same way but carries
# the backward pass in FP64.  Over four layers and 4096 records that leaves a
# few parts per thousand of relative error per layer (measured on a GB300:
# at most 1.8e-3 relative, cosine above 0.999998, in the first layer; less
# in the later ones).
GRAD_COS = 0.99995
GRAD_REL = 5e-3


@pytest.mark.parametrize("case", ["kl_host", "kl", "chi2", "chi2_oneblob"])
def test_gradient_matches_oracle(gpu_lib, case):
    """kl_host: pt_debug_nn_grad (T summed on the host, KL weights, c in
    [0.1, 0.9]).  kl / chi2: pt_debug_nn_grad_ex, the renderer's own step
    (T summed, and squared for chi-square, on the device) with the renderer's
    default BSDF-fraction range [0.3, 0.9]; chi2 is the renderer's default
    divergence.  chi2_oneblob: the same with the one-blob input encoding."""
    from cpppt import lib
    from oracle import nn_oracle
    w = random_weights(4)
    rec = _grad_records(4096, 3)
    if case == "kl_host":
        loss, g = lib.nn_grad(w, LO, HI, rec)
        rloss, rg = nn_oracle.loss_and_grad(w, LO, HI, rec)
    else:
        enc = 1 if case.endswith("oneblob") else 0
        dname = case.split("_")[0]
        div = lib.NN_CHI2 if dname == "chi2" else lib.NN_KL
        loss, g = lib.nn_grad_step(w, LO, HI, rec, divergence=div, c_lo=0.3, c_hi=0.9, encoding=enc)
        rloss, rg = nn_oracle.loss_and_grad(w, LO, HI, rec, divergence=dname, c_lo=0.3, c_hi=0.9, encoding=enc)
    assert abs(loss - rloss) < 2e-3 * max(1.0, abs(rloss)), (loss, rloss)
    off = 0
    for i, o in [(64, 64), (64, 64), (64, 64), (64, 48)]:
        a, b = g[off:off + i * o], rg[off:off + i * o]
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
        rel = float(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))
        assert cos > GRAD_COS and rel < GRAD_REL, (off, cos, rel)
        off += i * o


def test_chi2_differs_from_kl(gpu_lib):
    """The two divergences weigh the same records differently, so their
    gradients must differ by far more than the rounding error above (the
    chi-square path is really taken)."""
    from cpppt import lib
    w = random_weights(4)
    rec = _grad_records(2048, 8)
    _, gk = lib.nn_grad_step(w, LO, HI, rec, divergence=lib.NN_KL)
    _, gc = lib.nn_grad_step(w, LO, HI, rec, divergence=lib.NN_CHI2)
    diff = float(np.linalg.norm(gk / np.linalg.norm(gk) - gc / np.linalg.norm(gc)))
    assert diff > 10 * GRAD_REL, diff


@pytest.mark.parametrize("encoding", [0, 1], ids=["freq", "oneblob"])
def test_guided_render_converges_to_plain(gpu_lib, encoding):
    """Both estimators are unbiased (PT_FLAG_UNBIASED_MIS for plain PT), so
    after training the guided image must match the plain one statistically,
    with either input encoding of the guide."""
    from cpppt import scenes
    from cpppt.lib import FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, GpuScene
    from tests.test_gpu_render import check_z, tile_means, ztest
    sc = scenes.slit_room(seed=4, n_boxes=60, box_subdiv=2, width=64, height=32)
    gs = GpuScene(sc)
    cfg = gs.nn_configure(batch=1 << 14, encoding=encoding)
    assert cfg["batch"] == 1 << 14 and cfg["encoding"] == encoding
    for k in range(6):  # train the guide
        gs.render(256, max_depth=12, seed=1000 + k, mode=MODE_NN)
    st = gs.nn_stats()
    assert st["steps"] >= 4, st
    R, tile = 8, 16
    g = np.stack([gs.render(256, max_depth=12, seed=50 + r, mode=MODE_NN) for r in range(R)])
    p = np.stack([gs.render(256, max_depth=12, seed=90 + r, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
                  for r in range(R)])
    assert np.isfinite(g).all() and np.isfinite(p).all()
    check_z(ztest(tile_means(g, tile), tile_means(p, tile)), max_abs=6.0, frac3=0.1)


def test_trained_guide_lowers_variance(gpu_lib):
    """What the trained network gains over the method without it: on the
    occluded-light room (1000 boxes, light through a slit, 640x360), after
    online training the frozen guide's per-sample variance at depth 3
    (direct light and two bounces of indirect light) is clearly below plain
    PT's, with the same estimator otherwise (PT_FLAG_UNBIASED_MIS)."""
    from cpppt import scenes
    from cpppt.lib import FLAG_NN_FREEZE, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, GpuScene
    sc = scenes.slit_room(seed=4, n_boxes=1000, box_subdiv=4, width=640, height=360)
    gs = GpuScene(sc)
    gs.nn_reset(11)
    gs.nn_configure(bsdf_frac_min=0.1)
    # training is not deterministic (gradient sums use atomics): after 200
    # renders the variance ratio below spread over 0.77-0.86 on repeated runs,
    # after 400 over 0.57-0.71
    for k in range(400):
        gs.render(4, max_depth=12, seed=3000 + k, mode=MODE_NN)
    assert gs.nn_stats()["steps"] >= 400

    def rel_var(mode, flags, seed0, R=8, S=16):
        x = np.stack([gs.render(S, max_depth=3, seed=seed0 + r, mode=mode, flags=flags) for r in range(R)])
        m = x.mean(0)
        return float(np.mean(x.var(0, ddof=1) * S / (m ** 2 + 1e-2))), float(m.mean())

    v_plain, m_plain = rel_var(MODE_MIS, FLAG_UNBIASED_MIS, 100)
    v_nn, m_nn = rel_var(MODE_NN, FLAG_NN_FREEZE, 200)
    assert abs(m_nn - m_plain) < 0.03 * m_plain, (m_nn, m_plain)  # same image
    assert v_nn < 0.85 * v_plain, (v_nn, v_plain)


def test_guide_settings_are_checked(gpu_lib):
    """pt_nn_configure: the defaults, the accepted ranges, and every
    out-of-range value refused with the previous settings kept."""
    from cpppt import scenes
    from cpppt.lib import NN_CHI2, NN_ENC_FREQ, NN_ENC_ONEBLOB, GpuScene, PtError
    gs = GpuScene(scenes.cornell(8, 8))
    cfg = gs.nn_config()
    assert cfg["batch"] == 65536 and cfg["steps_per_round"] == 16 and cfg["divergence"] == NN_CHI2
    assert abs(cfg["learning_rate"] - 3e-3) < 1e-9 and abs(cfg["bsdf_frac_min"] - 0.3) < 1e-7
    assert cfg["encoding"] == NN_ENC_FREQ and cfg["passes"] == 1
    assert gs.nn_configure(steps_per_round=64, batch=1024)["steps_per_round"] == 64
    assert gs.nn_configure(encoding=NN_ENC_ONEBLOB)["encoding"] == NN_ENC_ONEBLOB
    assert gs.nn_configure(passes=8)["passes"] == 8
    gs.nn_configure(**cfg)
    for bad in (dict(steps_per_round=65), dict(steps_per_round=0), dict(batch=1023), dict(batch=262145),
                dict(bsdf_frac_min=0.05), dict(bsdf_frac_min=0.9, bsdf_frac_max=0.8), dict(learning_rate=0.0),
                dict(divergence=2), dict(encoding=2), dict(encoding=-1), dict(passes=0), dict(passes=9)):
        with pytest.raises(PtError):
            gs.nn_configure(**bad)
        assert gs.nn_config() == cfg


def test_passes_take_several_steps_per_batch(gpu_lib):
    """passes = 3: every batch of records is used for three Adam steps (the
    chi-square targets prepared once), so the step count is three times the
    batches trained on, and the guided image stays finite and lit."""
    from cpppt import scenes
    from cpppt.lib import MODE_NN, GpuScene
    gs = GpuScene(scenes.slit_room(seed=4, n_boxes=60, box_subdiv=2, width=64, height=32))
    gs.nn_configure(batch=1024, passes=3, steps_per_round=8)
    for k in range(4):
        img = gs.render(64, max_depth=12, seed=500 + k, mode=MODE_NN)
    st = gs.nn_stats()
    batches = st["records"] / 1024
    assert batches >= 4 and batches == int(batches), st
    assert st["steps"] == 3 * batches, st
    assert np.isfinite(img).all() and img.mean() > 0
