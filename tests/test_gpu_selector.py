"""Selector network kernels against a plain PyTorch FP32 reference of the
same ops (dense layer forward / backward, softmax cross-entropy, masked
squared error, Adam), a short training run, and labelling of one matrix."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("B,i,o,relu", [(1, 5, 3, 0), (37, 140, 256, 1), (128, 256, 256, 1), (300, 256, 18, 0)])
def test_linear_forward_backward_match_torch(B, i, o, relu):
    import torch
    from sspmv_gb300._lib import call
    g = torch.Generator(device="cuda").manual_seed(B + i)
    x = torch.randn(B, i, device="cuda", generator=g)
    W = torch.randn(o, i, device="cuda", generator=g) * 0.1
    b = torch.randn(o, device="cuda", generator=g)
    y = torch.empty(B, o, device="cuda")
    call("sspmv_nn_linear_forward", B, i, o, _p(x), i, _p(W), _p(b), relu, _p(y), o, _s())
    ref = x @ W.T + b
    if relu:
        ref = torch.relu(ref)
    torch.testing.assert_close(y, ref, rtol=1e-4, atol=1e-4)
    dy = torch.randn(B, o, device="cuda", generator=g)
    dy_ref = dy * (ref > 0) if relu else dy
    dx = torch.empty(B, i, device="cuda")
    dW = torch.empty(o, i, device="cuda")
    db = torch.empty(o, device="cuda")
    call("sspmv_nn_linear_backward", B, i, o, _p(x), i, _p(W), _p(y), relu, _p(dy), o, _p(dx), i, _p(dW), _p(db),
         _s())
    torch.testing.assert_close(dW, dy_ref.T @ x, rtol=1e-4, atol=1e-3)
    torch.testing.assert_close(db, dy_ref.sum(0), rtol=1e-4, atol=1e-3)
    torch.testing.assert_close(dx, dy_ref @ W, rtol=1e-4, atol=1e-3)


def test_losses_and_adam_match_torch():
    import torch
    from sspmv_gb300._lib import call
    g = torch.Generator(device="cuda").manual_seed(3)
    B, Cc = 50, 9
    out = torch.randn(B, 2 * Cc, device="cuda", generator=g)
    lab = torch.randint(0, Cc, (B,), device="cuda", generator=g, dtype=torch.int32)
    lab[3] = -1
    dout = torch.zeros_like(out)
    lrow = torch.empty(B, device="cuda")
    call("sspmv_nn_softmax_xent", B, Cc, _p(out), 2 * Cc, _p(lab), _p(dout), 2 * Cc, _p(lrow), _s())
    z = out[:, :Cc].clone().requires_grad_(True)
    keep = lab >= 0
    lref = torch.nn.functional.cross_entropy(z[keep], lab[keep].long(), reduction="none")
    (lref.sum() / B).backward()
    torch.testing.assert_close(lrow[keep], lref.detach(), rtol=1e-5, atol=1e-5)
    assert lrow[3].item() == 0.0
    torch.testing.assert_close(dout[:, :Cc], z.grad, rtol=1e-5, atol=1e-6)
    tgt = torch.randn(B, Cc, device="cuda", generator=g)
    mask = (torch.rand(B, Cc, device="cuda", generator=g) > 0.3).float()
    cnt = float(mask.sum().item())
    mrow = torch.empty(B, device="cuda")
    base = out.data_ptr() + 4 * Cc
    call("sspmv_nn_masked_mse", B, Cc, C.c_void_p(base), 2 * Cc, _p(tgt), _p(mask), 0.5, cnt,
         C.c_void_p(dout.data_ptr() + 4 * Cc), 2 * Cc, _p(mrow), _s())
    p = out[:, Cc:].clone().requires_grad_(True)
    lm = (((p - tgt) ** 2) * mask).sum() / cnt
    (0.5 * lm).backward()
    torch.testing.assert_close(mrow.sum(), lm.detach(), rtol=1e-5, atol=1e-6)
    torch.testing.assert_close(dout[:, Cc:], p.grad, rtol=1e-5, atol=1e-7)
    # Adam: three steps against torch.optim.Adam with L2 weight decay
    w = torch.randn(1000, device="cuda", generator=g)
    w_ref = w.clone().requires_grad_(True)
    opt = torch.optim.Adam([w_ref], lr=1e-2, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-3)
    m = torch.zeros_like(w)
    v = torch.zeros_like(w)
    for step in range(1, 4):
        grad = torch.randn(1000, device="cuda", generator=g)
        call("sspmv_nn_adam", 1000, _p(w), _p(grad), _p(m), _p(v), 1e-2, 0.9, 0.999, 1e-8, step, 1e-3, _s())
        opt.zero_grad()
        w_ref.grad = grad.clone()
        opt.step()
    torch.testing.assert_close(w, w_ref.detach(), rtol=1e-5, atol=1e-6)


def test_mlp_learns_a_separable_rule():
    """A rule the features determine (format = bucket of feature 0) is
    learned to near-zero regret."""
    from sspmv_gb300 import selector as S
    rng = np.random.default_rng(0)
    n = 600
    raw = np.zeros((n, 66))
    raw[:, 0] = rng.normal(size=n)
    raw[:, 1:8] = 0.1 * rng.normal(size=(n, 7))
    bucket = np.digitize(raw[:, 0], [-0.5, 0.5])  # 0, 1, 2
    fmts = [S.LABELS.index("ell"), S.CSR_LABEL, S.LABELS.index("sell_c_sigma")]
    times = np.full((n, S.NUM_CLASSES), 3.0)
    times[:, S.CSR_LABEL] = 2.0
    for k in range(n):
        times[k, fmts[bucket[k]]] = 1.0
    ds = S.Dataset(raw, times, np.arange(n))
    net, res = S.evaluate(ds, train_frac=0.8, epochs=120)
    # misses only near the two thresholds (480 training matrices)
    assert res["mean_regret"] < 0.2 and res["exact_pick_rate"] > 0.85, res
    assert res["mean_regret"] < res["csr_mean_regret"] / 3, res


def test_label_matrix_times_every_feasible_format():
    from sspmv_gb300 import selector as S
    from sspmv_gb300 import synth
    A = synth.generate(synth.banded(50000, (0, 1, -1, 4, -4)), 3)
    rec = S.label_matrix(A)
    assert len(rec["raw"]) == 66 and rec["raw"][43] == 5
    for f in ("csr", "coo", "ell", "sell", "sell_c_sigma", "sell_c_R", "dia", "csr5"):
        assert rec["times"][f] is not None and rec["times"][f] > 0, f


def test_packaged_selector_regret_on_held_out_matrices():
    """The packaged model (trained on the first 1,600 of the packaged 2,000
    GPU-labelled matrices, seed-0 split) picks formats on the other 400 with
    far lower regret than always using CSR."""
    from sspmv_gb300 import selector as S
    ds = S.load_dataset(S.PACKAGE_DATA / "selector_dataset.npz")
    perm = np.random.default_rng(0).permutation(len(ds.ids))
    te = perm[1600:]
    net = S.load_model(S.PACKAGE_DATA / "selector_model.npz")
    picks = S.choose(net, ds.raw[te], np.isfinite(ds.times[te]))
    r = S.regret(ds.times[te], picks)
    assert r["mean_regret"] < 0.05 and r["mean_regret"] < r["csr_mean_regret"] / 3, r
