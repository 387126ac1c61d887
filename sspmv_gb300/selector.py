"""Format selector: GPU features -> FP32 multilayer perceptron -> format.

The reference's SmartAdpter trains Keras networks offline on features its
Get_features program writes (src/sparse_features.cpp) and on labels from its
CPU benchmark runs (script/write_label.py:63-75: COO 0, CSR 1, DIA 2, ELL 3,
S-ELL 4, S-ELL-sigma 5, S-ELL-R 6, CSR5 7, BSR 8).  Here everything runs on
the GPU through the library:
  - features: sspmv_csr_features (62 values, T x T tiles) and
    sspmv_csr_grx_features (GrX, X = 4), each value also as a signed log,
    standardised with the training set's mean and deviation;
  - labels: every format converted with a few parameter sets and timed on the
    GPU (L2 flushed, CUDA events), the fastest (format, parameters) kept;
  - network: inputs -> 256 -> 256 (ReLU) -> 9 class logits + 9 predicted
    log(time_format / time_csr) values, trained with the library's own dense
    layer, loss and Adam kernels (sspmv_nn_*), PyTorch tensors only holding
    the memory;
  - decision: the format with the best predicted time among those feasible
    for the matrix, plain CSR when no format is predicted faster than CSR
    (rule "time"; rule "class" takes the most likely class instead).
Regret of a pick = its measured time / the fastest measured time - 1.
"""
from __future__ import annotations

import json
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import _lib, synth
from ._lib import call
from .synth import HostCSR

LABELS = ["coo", "csr", "dia", "ell", "sell", "sell_c_sigma", "sell_c_R", "csr5", "bsr"]
NUM_CLASSES = len(LABELS)
CSR_LABEL = LABELS.index("csr")
TILES = 2048
GROUP = 4
NUM_DIAGS = 43  # index of num_diags in the feature vector

# Parameter sets tried per format when labelling (library defaults first).
LABEL_CANDIDATES = {
    "csr": [("kernel", 0, 0), ("kernel", 2, 0), ("kernel", 1, 2), ("kernel", 1, 8), ("kernel", 1, 32)],
    "coo": [("kernel", 0, 0), ("kernel", 1, 0)],
    "ell": [{}],
    "sell": [dict(chunkwidth=8, alignment=0), dict(chunkwidth=32, alignment=0)],
    "sell_c_sigma": [dict(slicewidth=0, chunkwidth=0, alignment=0), dict(slicewidth=256, chunkwidth=8, alignment=0),
                     dict(slicewidth=4096, chunkwidth=32, alignment=0)],
    "sell_c_R": [dict(chunkwidth=8, alignment=0), dict(chunkwidth=32, alignment=0)],
    "dia": [{}],
    "csr5": [dict(sigma=0, omega=0), dict(sigma=16, omega=32)],
    "bsr": [dict(blockDimRow=2, blockDimCol=2), dict(blockDimRow=4, blockDimCol=4), dict(blockDimRow=8, blockDimCol=8)],
}


# ------------------------------------------------------------ matrix mix --
def _banded_params(rng, n, r):
    d = int(np.clip(round(r), 1, 32))
    spread = max([8, 512, max(16, n // 8)][rng.integers(0, 3)], d)
    offs = {0}
    while len(offs) < d:
        offs.add(int(rng.integers(-spread, spread + 1)))
    return synth.banded(n, tuple(sorted(offs)))


def _family_params(rng, fam, n, r):
    if fam == "banded":
        return _banded_params(rng, n, r)
    if fam == "powerlaw":
        return synth.powerlaw(n, float(rng.uniform(1.6, 2.6)), float(r), min(50000, n),
                              float(rng.choice([0.0, 0.0, 0.05, 0.2])))
    if fam == "block":
        b = int(rng.choice([2, 4, 8]))
        return synth.block(n, b, max(1, int(r * n / (b * b))))
    return synth.uniform(n, int(np.clip(round(r), 1, min(n, 2000))), float(rng.choice([0.0, 0.0, 0.1])))


def dataset_spec(i: int, seed: int = 0) -> dict:
    """Parameters of dataset matrix i: family (the four synthetic families or
    a mixture of two stacked row halves), N log-uniform in [1e4, 2e6], target
    nnz log-uniform in [5e4, 2e7]."""
    rng = np.random.default_rng([seed, i])
    fam = ["banded", "powerlaw", "block", "uniform", "mix"][int(rng.integers(0, 5))]
    n = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
    nnz = float(np.exp(rng.uniform(np.log(5e4), np.log(2e7))))
    r = float(np.clip(nnz / n, 1.0, 1000.0))
    return {"i": i, "family": fam, "n": n, "r": r, "seed": seed}


def dataset_matrix(spec: dict, dtype=np.float64) -> HostCSR:
    rng = np.random.default_rng([spec["seed"], spec["i"], 1])
    n, r = spec["n"], spec["r"]
    if spec["family"] != "mix":
        if spec["family"] == "block":
            n -= n % 8
        return synth.generate(_family_params(rng, spec["family"], n, r), 1000 + spec["i"], dtype)
    fa, fb = rng.choice(["banded", "powerlaw", "block", "uniform"], 2, replace=False)
    n -= n % 16
    top = synth.generate(_family_params(rng, fa, n, r), 2000 + spec["i"], dtype)
    bot = synth.generate(_family_params(rng, fb, n, r), 3000 + spec["i"], dtype)
    h = n // 2
    rp = np.concatenate([top.row_offset[:h + 1],
                         top.row_offset[h] + bot.row_offset[h + 1:] - bot.row_offset[h]]).astype(np.int32)
    ci = np.concatenate([top.col_index[:top.row_offset[h]], bot.col_index[bot.row_offset[h]:]])
    cv = np.concatenate([top.values[:top.row_offset[h]], bot.values[bot.row_offset[h]:]])
    return HostCSR(n, n, rp, ci, cv)


# --------------------------------------------------------------- features --
def raw_features(csr) -> np.ndarray:
    """62 MTX features (T = 2048) and 4 GrX features (X = 4) of a device CSR."""
    from . import lespmv as L
    F = L.features(csr, TILES)
    G = L.grx_features(csr, TILES, GROUP)
    return np.concatenate([F, G])


def model_inputs(raw: np.ndarray) -> np.ndarray:
    """Raw features and their signed logs (rows = matrices)."""
    raw = np.atleast_2d(np.asarray(raw, np.float64))
    # symmetry ratios are 0/0 for matrices without off-diagonal entries, and
    # value maxima start at -DBL_MAX when a matrix has no such entry
    raw = np.clip(np.nan_to_num(raw, nan=0.0, posinf=1e30, neginf=-1e30), -1e30, 1e30)
    return np.concatenate([raw, np.sign(raw) * np.log1p(np.abs(raw))], axis=1)


# ---------------------------------------------------------------- labels --
def _time_ms(M, x, y, flush, reps=3):
    from .autotune import time_spmv
    return time_spmv(M, x, y, reps=reps, warmup=1, flush=flush)


def label_matrix(A: HostCSR, flush=None) -> dict:
    """Measured best time (ms) and parameters of every format on A (None when
    the format is infeasible), and the raw features."""
    from .autotune import L2Flush
    import torch
    from . import lespmv as L
    csr = L.csr_from_host(A)
    x = torch.from_numpy(synth.vector(A.num_cols, 0, A.values.dtype)).cuda()
    y = torch.zeros(A.num_rows, dtype=x.dtype, device="cuda")
    if flush is None:
        flush = L2Flush("cuda")
    out = {"times": {}, "params": {}}
    t0 = time.perf_counter()
    out["raw"] = raw_features(csr).tolist()
    out["feature_ms"] = (time.perf_counter() - t0) * 1e3
    for fmt in LABELS:
        best = None
        for cand in LABEL_CANDIDATES[fmt]:
            M = None
            try:
                if isinstance(cand, tuple):
                    base = csr if fmt == "csr" else L.csr_to_coo(csr)
                    M = base
                    M.set_kernel(cand[1], cand[2])
                    ms = _time_ms(M, x, y, flush)
                    rec = {"kernel_flag": cand[1], "param": cand[2]}
                    if fmt != "csr":
                        M.delete()
                else:
                    if fmt == "ell" and not L.feasible_host("ell", A)[0]:
                        continue
                    if fmt == "dia":
                        nd = out["raw"][NUM_DIAGS]
                        if nd > 10240 or nd * A.num_rows > 8 * max(A.nnz, 1):
                            continue
                    if fmt == "bsr":
                        nb = L.count_blocks(csr, cand["blockDimRow"], cand["blockDimCol"])
                        if nb * cand["blockDimRow"] * cand["blockDimCol"] > 4 * max(A.nnz, 1):
                            continue
                    M = getattr(L, f"csr_to_{fmt}")(csr, **cand)
                    ms = _time_ms(M, x, y, flush)
                    rec = dict(cand)
                    M.delete()
            except _lib.SSPMVError:
                if M is not None and M is not csr:
                    M.delete()
                continue
            if best is None or ms < best[0]:
                best = (ms, rec)
        out["times"][fmt] = best[0] if best else None
        out["params"][fmt] = best[1] if best else None
    csr.set_kernel(0, 0)
    csr.delete()
    return out


def build_dataset(path: str | Path, count: int, start: int = 0, seed: int = 0, log=None) -> None:
    """Appends label records of matrices start .. start+count-1 to a JSONL
    file (matrices already present are skipped, so runs can be resumed)."""
    from .autotune import L2Flush
    import torch
    log = log or (lambda *a: None)
    path = Path(path)
    done = set()
    if path.exists():
        for ln in path.read_text().splitlines():
            if ln.strip():
                done.add(json.loads(ln)["i"])
    flush = L2Flush("cuda")
    with open(path, "a") as f:
        for i in range(start, start + count):
            if i in done:
                continue
            spec = dataset_spec(i, seed)
            t0 = time.perf_counter()
            A = dataset_matrix(spec, np.float64)
            rec = label_matrix(A, flush)
            rec.update(spec)
            rec.update({"num_rows": A.num_rows, "nnz": A.nnz, "label_s": time.perf_counter() - t0})
            f.write(json.dumps(rec) + "\n")
            f.flush()
            best = min((t, k) for k, t in rec["times"].items() if t is not None)
            log(f"[dataset] {i} {spec['family']} n={A.num_rows} nnz={A.nnz} best={best[1]} "
                f"{rec['label_s']:.2f}s")


@dataclass
class Dataset:
    raw: np.ndarray        # matrices x 66
    times: np.ndarray      # matrices x 9 (ms, inf = infeasible)
    ids: np.ndarray

    @property
    def labels(self) -> np.ndarray:
        return np.argmin(self.times, axis=1).astype(np.int32)


PACKAGE_DATA = Path(__file__).resolve().parent / "data"


def load_dataset(paths) -> Dataset:
    """Labelled matrices from JSONL files written by build_dataset, or from
    an .npz with raw / times / ids arrays (the packaged measured dataset,
    sspmv_gb300/data/selector_dataset.npz)."""
    if isinstance(paths, (str, Path)) and str(paths).endswith(".npz"):
        d = np.load(paths)
        return Dataset(np.asarray(d["raw"]), np.asarray(d["times"]), np.asarray(d["ids"]))
    recs = {}
    for p in ([paths] if isinstance(paths, (str, Path)) else paths):
        for ln in Path(p).read_text().splitlines():
            if ln.strip():
                r = json.loads(ln)
                recs[r["i"]] = r
    ids = np.array(sorted(recs))
    raw = np.array([recs[i]["raw"] for i in ids])
    times = np.array([[recs[i]["times"][f] if recs[i]["times"][f] is not None else np.inf for f in LABELS]
                      for i in ids])
    return Dataset(raw, times, ids)


# ---------------------------------------------------------------- network --
class MLP:
    """inputs -> 256 -> 256 -> 18 (9 logits, 9 log time ratios), FP32 on the
    GPU; every product, loss and update runs in the library's sspmv_nn_*
    kernels."""

    def __init__(self, n_in: int, hidden: int = 256, seed: int = 0):
        import torch
        g = torch.Generator().manual_seed(seed)
        dims = [n_in, hidden, hidden, 2 * NUM_CLASSES]
        self.dims = dims
        self.W, self.b = [], []
        for a, o in zip(dims[:-1], dims[1:]):
            w = (torch.rand(o, a, generator=g) * 2 - 1) * (6.0 / (a + o)) ** 0.5
            self.W.append(w.float().cuda().contiguous())
            self.b.append(torch.zeros(o, device="cuda"))
        self.params = self.W + self.b
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.grads = [torch.zeros_like(p) for p in self.params]
        self.step = 0
        self.mean = None
        self.std = None

    @staticmethod
    def _p(t):
        return C_void(t.data_ptr())

    def forward(self, X):
        """X: batch x n_in float32 CUDA tensor -> list of layer outputs."""
        import torch
        acts = [X]
        s = _stream()
        for li, (W, b) in enumerate(zip(self.W, self.b)):
            o, a = W.shape
            y = torch.empty(X.shape[0], o, device="cuda")
            relu = 1 if li < len(self.W) - 1 else 0
            call("sspmv_nn_linear_forward", X.shape[0], a, o, self._p(acts[-1]), a, self._p(W), self._p(b), relu,
                 self._p(y), o, s)
            acts.append(y)
        return acts

    def train_step(self, X, labels, target, mask, lr=1e-3, wd=1e-5, reg_weight=1.0) -> float:
        import torch
        B = X.shape[0]
        s = _stream()
        acts = self.forward(X)
        out = acts[-1]
        dout = torch.zeros_like(out)
        lc = torch.empty(B, device="cuda")
        lr_rows = torch.empty(B, device="cuda")
        call("sspmv_nn_softmax_xent", B, NUM_CLASSES, self._p(out), out.shape[1], self._p(labels), self._p(dout),
             out.shape[1], self._p(lc), s)
        cnt = float(max(1.0, mask.sum().item()))
        call("sspmv_nn_masked_mse", B, NUM_CLASSES, C_void(out.data_ptr() + 4 * NUM_CLASSES), out.shape[1],
             self._p(target), self._p(mask), float(reg_weight), cnt, C_void(dout.data_ptr() + 4 * NUM_CLASSES),
             out.shape[1], self._p(lr_rows), s)
        dy = dout
        nl = len(self.W)
        for li in reversed(range(nl)):
            W = self.W[li]
            o, a = W.shape
            x = acts[li]
            dx = torch.empty(B, a, device="cuda") if li > 0 else None
            call("sspmv_nn_linear_backward", B, a, o, self._p(x), a, self._p(W), self._p(acts[li + 1]),
                 1 if li < nl - 1 else 0, self._p(dy), o, self._p(dx) if dx is not None else None, a,
                 self._p(self.grads[li]), self._p(self.grads[nl + li]), s)
            dy = dx
        self.step += 1
        for p, g, m, v in zip(self.params, self.grads, self.m, self.v):
            call("sspmv_nn_adam", p.numel(), self._p(p), self._p(g), self._p(m), self._p(v), float(lr), 0.9, 0.999,
                 1e-8, self.step, float(wd), s)
        return float(lc.mean().item() + lr_rows.sum().item())

    def predict(self, X):
        out = self.forward(X)[-1]
        return out[:, :NUM_CLASSES], out[:, NUM_CLASSES:]

    def state(self) -> dict:
        d = {f"W{i}": w.cpu().numpy() for i, w in enumerate(self.W)}
        d.update({f"b{i}": b.cpu().numpy() for i, b in enumerate(self.b)})
        d["mean"], d["std"] = self.mean, self.std
        return d

    @classmethod
    def from_state(cls, d: dict) -> "MLP":
        import torch
        net = cls(int(d["W0"].shape[1]), int(d["W0"].shape[0]))
        for i in range(len(net.W)):
            net.W[i].copy_(torch.from_numpy(np.asarray(d[f"W{i}"], np.float32)))
            net.b[i].copy_(torch.from_numpy(np.asarray(d[f"b{i}"], np.float32)))
        net.mean, net.std = np.asarray(d["mean"]), np.asarray(d["std"])
        return net


def C_void(v):
    import ctypes
    return ctypes.c_void_p(int(v)) if v is not None else None


def _stream():
    import ctypes
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def targets_from_times(times: np.ndarray):
    """log(time / time_csr) per format and the feasibility mask."""
    csr = times[:, CSR_LABEL:CSR_LABEL + 1]
    mask = np.isfinite(times).astype(np.float32)
    t = np.where(mask > 0, np.log(np.where(mask > 0, times, 1.0) / csr), 0.0).astype(np.float32)
    return t, mask


def train(ds: Dataset, train_idx, epochs: int = 400, batch: int = 128, lr: float = 2e-3, seed: int = 0,
          log=None) -> MLP:
    import torch
    log = log or (lambda *a: None)
    X = model_inputs(ds.raw[train_idx])
    mean, std = X.mean(0), X.std(0) + 1e-6
    Xn = torch.from_numpy(((X - mean) / std).astype(np.float32)).cuda()
    lab = torch.from_numpy(ds.labels[train_idx]).cuda()
    t, mk = targets_from_times(ds.times[train_idx])
    T = torch.from_numpy(t).cuda()
    Mk = torch.from_numpy(mk).cuda()
    net = MLP(X.shape[1], seed=seed)
    net.mean, net.std = mean, std
    rng = np.random.default_rng(seed)
    n = len(train_idx)
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(n)).cuda()
        tot = 0.0
        for s in range(0, n, batch):
            idx = perm[s:s + batch]
            step_lr = lr * 0.5 * (1 + np.cos(np.pi * ep / epochs))
            tot += net.train_step(Xn[idx].contiguous(), lab[idx].contiguous(), T[idx].contiguous(),
                                  Mk[idx].contiguous(), lr=step_lr)
        if ep % 50 == 0 or ep == epochs - 1:
            log(f"[selector] epoch {ep} loss {tot / max(1, (n + batch - 1) // batch):.4f}")
    return net


def choose(net: MLP, raw: np.ndarray, feasible: np.ndarray | None = None, rule: str = "time") -> np.ndarray:
    """Format label per matrix.  rule "class": the most likely feasible class,
    kept only when the time head does not predict it slower than CSR
    (otherwise CSR).  rule "time": the best predicted time among feasible
    formats, CSR unless a format is predicted faster."""
    import torch
    X = (model_inputs(raw) - net.mean) / net.std
    logits, tpred = net.predict(torch.from_numpy(X.astype(np.float32)).cuda())
    tp = tpred.cpu().numpy().astype(np.float64)
    lg = logits.cpu().numpy().astype(np.float64)
    if feasible is not None:
        tp = np.where(feasible, tp, np.inf)
        lg = np.where(feasible, lg, -np.inf)
    tp[:, CSR_LABEL] = 0.0
    if rule == "time":
        return np.argmin(tp, axis=1)
    picks = np.argmax(lg, axis=1)
    slower = tp[np.arange(len(picks)), picks] > 0.0
    return np.where(slower, CSR_LABEL, picks)


def regret(times: np.ndarray, picks: np.ndarray) -> dict:
    best = times.min(axis=1)
    t = times[np.arange(len(picks)), picks]
    t = np.where(np.isfinite(t), t, times[:, CSR_LABEL])  # an infeasible pick falls back to CSR
    r = t / best - 1.0
    csr_r = times[:, CSR_LABEL] / best - 1.0
    return {"mean_regret": float(r.mean()), "median_regret": float(np.median(r)), "p90_regret": float(np.quantile(r, 0.9)),
            "exact_pick_rate": float((r <= 1e-12).mean()), "csr_mean_regret": float(csr_r.mean()),
            "csr_p90_regret": float(np.quantile(csr_r, 0.9)),
            "time_ratio_vs_best": float(t.sum() / best.sum()),
            "csr_time_ratio_vs_best": float(times[:, CSR_LABEL].sum() / best.sum())}


def evaluate(ds: Dataset, train_frac: float = 0.8, seed: int = 0, epochs: int = 400, log=None):
    """Train on a seeded train_frac split, report regret on the rest."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(len(ds.ids))
    ntr = int(round(train_frac * len(perm)))
    tr, te = perm[:ntr], perm[ntr:]
    t0 = time.perf_counter()
    net = train(ds, tr, epochs=epochs, seed=seed, log=log)
    train_s = time.perf_counter() - t0
    feas = np.isfinite(ds.times[te])
    picks = choose(net, ds.raw[te], feas, "time")
    res = regret(ds.times[te], picks)
    res["class_rule"] = regret(ds.times[te], choose(net, ds.raw[te], feas, "class"))
    res.update({"train": int(ntr), "test": int(len(te)), "train_s": round(train_s, 2),
                "label_hist": np.bincount(ds.labels, minlength=NUM_CLASSES).tolist(),
                "pick_hist": np.bincount(picks, minlength=NUM_CLASSES).tolist()})
    return net, res


def save_model(net: MLP, path: str | Path, params: dict | None = None) -> None:
    d = net.state()
    d["format_params"] = np.frombuffer(json.dumps(params or {}).encode(), np.uint8)
    np.savez(path, **d)


def load_model(path: str | Path) -> MLP:
    d = dict(np.load(path))
    d.pop("format_params", None)
    return MLP.from_state(d)


MAX_ROW = 7     # feature index: longest row
NUM_ROWS = 0
NUM_NNZ = 2


def feasible_from_features(raw: np.ndarray) -> np.ndarray:
    """Formats that can be built for each matrix, from its features alone
    (the labelling rules: ELL padding within 4x, DIA within 10240 diagonals
    and 8x padding).  BSR is decided by its converter at load time."""
    raw = np.atleast_2d(raw)
    m, nnz = raw[:, NUM_ROWS], np.maximum(raw[:, NUM_NNZ], 1)
    f = np.ones((len(raw), NUM_CLASSES), bool)
    f[:, LABELS.index("ell")] = raw[:, MAX_ROW] * m <= 4 * nnz
    nd = raw[:, NUM_DIAGS]
    f[:, LABELS.index("dia")] = (nd <= 10240) & (nd * m <= 8 * nnz)
    return f


def common_params(paths) -> dict:
    """Most frequent best parameter set per format in labelled data."""
    from collections import Counter
    cnt = {f: Counter() for f in LABELS}
    for p in ([paths] if isinstance(paths, (str, Path)) else paths):
        for ln in Path(p).read_text().splitlines():
            if ln.strip():
                r = json.loads(ln)
                for f, prm in r["params"].items():
                    if prm is not None:
                        cnt[f][json.dumps(prm, sort_keys=True)] += 1
    return {f: json.loads(c.most_common(1)[0][0]) for f, c in cnt.items() if c}


def pack_dataset(paths, out) -> None:
    """Writes labelled JSONL records as one .npz: raw features, times per
    format (inf: infeasible), matrix ids, family, rows, nonzeros and the most
    frequent best parameters per format (JSON bytes) -- the layout of
    sspmv_gb300/data/selector_dataset.npz."""
    ds = load_dataset(paths)
    recs = {}
    for p in ([paths] if isinstance(paths, (str, Path)) else paths):
        for ln in Path(p).read_text().splitlines():
            if ln.strip():
                r = json.loads(ln)
                recs[r["i"]] = r
    fam = np.array([recs[int(i)]["family"] for i in ds.ids])
    rows = np.array([recs[int(i)]["num_rows"] for i in ds.ids], np.int64)
    nnz = np.array([recs[int(i)]["nnz"] for i in ds.ids], np.int64)
    params = np.frombuffer(json.dumps(common_params(paths)).encode(), np.uint8)
    np.savez(out, raw=ds.raw, times=ds.times, ids=ds.ids, family=fam, num_rows=rows, nnz=nnz,
             format_params=params)


class Selector:
    """A trained network and the parameter set it uses per format; picks the
    serving format of a device CSR matrix."""

    def __init__(self, path: str | Path):
        d = dict(np.load(path))
        self.params = json.loads(bytes(d.pop("format_params", np.zeros(2, np.uint8))).decode() or "{}")
        self.net = MLP.from_state(d)

    def pick(self, csr) -> tuple[str, dict | None]:
        raw = raw_features(csr)[None, :]
        fmt = LABELS[int(choose(self.net, raw, feasible_from_features(raw))[0])]
        return fmt, self.params.get(fmt)


def main(argv=None) -> None:
    """python -m sspmv_gb300.selector dataset --out FILE --count N [--start S]
       python -m sspmv_gb300.selector pack --data FILE [FILE...] --out DATASET.npz
       python -m sspmv_gb300.selector train --data FILE [FILE...] --model OUT.npz --report OUT.json"""
    import argparse
    import sys
    ap = argparse.ArgumentParser(prog="python -m sspmv_gb300.selector")
    sub = ap.add_subparsers(dest="cmd", required=True)
    d = sub.add_parser("dataset")
    d.add_argument("--out", required=True)
    d.add_argument("--count", type=int, default=2000)
    d.add_argument("--start", type=int, default=0)
    d.add_argument("--seed", type=int, default=0)
    d.add_argument("--budget-s", type=float, default=0.0, help="stop after this many seconds (0: no limit)")
    pk = sub.add_parser("pack", help="JSONL label files -> one .npz (the packaged dataset layout)")
    pk.add_argument("--data", nargs="+", required=True)
    pk.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", nargs="+", required=True)
    t.add_argument("--model", required=True)
    t.add_argument("--report", required=True)
    t.add_argument("--epochs", type=int, default=400)
    t.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    log = lambda *m: print(*m, file=sys.stderr, flush=True)  # noqa: E731
    if a.cmd == "dataset":
        t0 = time.perf_counter()
        step = 25
        for s in range(a.start, a.start + a.count, step):
            if a.budget_s and time.perf_counter() - t0 > a.budget_s:
                log(f"[dataset] budget reached before matrix {s}")
                break
            build_dataset(a.out, min(step, a.start + a.count - s), s, a.seed, log)
        return
    if a.cmd == "pack":
        pack_dataset(a.data, a.out)
        return
    ds = load_dataset(a.data[0] if len(a.data) == 1 and a.data[0].endswith(".npz") else a.data)
    net, res = evaluate(ds, 0.8, a.seed, a.epochs, log)
    res["matrices"] = int(len(ds.ids))
    if a.data[0].endswith(".npz"):
        params = json.loads(bytes(np.load(a.data[0])["format_params"]).decode())
    else:
        params = common_params(a.data)
    save_model(net, a.model, params)
    Path(a.report).write_text(json.dumps(res, indent=1) + "\n")
    log(json.dumps(res))


if __name__ == "__main__":
    main()
