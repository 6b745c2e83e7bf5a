"""Learned output-size predictor (no counterpart in the reference).

A small network (34 -> 64 -> 64 -> 1, ReLU, float32; forward, backward and
Adam are the library's own CUDA kernels, iso_mlp_*) predicts the triangles
(in units of LABEL_SCALE) of every 16^3-cell block of a volume at an
isovalue from the block's statistics (min, max, 32-bin histogram:
iso_block_stats, computed once per resident volume).  The labels are counts,
not their logarithms: the squared error then makes the output the
conditional mean, whose sum over blocks is unbiased (a log-space fit sums
geometric means and comes out low).  Summed over the blocks whose [min, max]
holds the isovalue (the others have no triangles), it sizes a mesh before any
pass over the volume: allocation and admission can then skip the exact count, and a
request whose mesh turns out too small falls back to the exact sizes, which
the extraction itself reports (ISO_ERR_CAPACITY).  The geometry never depends
on the network.

Training data follow the batched workload's distribution: volumes with
per-axis dimensions uniform in [32, 320], half Gaussian blobs and half value
noise, isovalues uniform in each field's [5th, 95th] percentile; labels are
the exact per-block triangle counts (iso_block_tris).

    python -m miniisosurface_gb300.predictor --out weights.f32
trains on 20,000 (volume, isovalue) pairs (500 volumes x 40 isovalues),
evaluates on held-out seeds and prints the metrics as JSON.
"""
import argparse
import ctypes as C
import json
import math
import time
from pathlib import Path

import numpy as np

from . import _lib
from .api import Context, _ptr, check, generate_blobs, generate_value_noise, load, make_grid

N_IN, N_HID = 34, 64
N_PARAMS = N_IN * N_HID + N_HID + N_HID * N_HID + 2 * N_HID + 1
LABEL_SCALE = 256.0  # triangles per unit of the network's output
WEIGHTS = Path(__file__).resolve().parent / "predictor_weights.f32"


def _stream(stream):
    import torch
    return C.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)


def block_count(dims):
    g = make_grid(dims)
    return int(load().iso_block_count(C.byref(g)))


def block_stats(volume, dims, stream=None):
    """(blocks, 34) float32 CUDA tensor: min, max, 32-bin histogram of each block (iso_block_stats)."""
    import torch
    nb = block_count(dims)
    out = torch.empty((max(nb, 1), N_IN), dtype=torch.float32, device=volume.device)
    g = make_grid(dims)
    check(load().iso_block_stats(_ptr(volume), C.byref(g), _ptr(out), _stream(stream)))
    return out[:nb]


def block_tris(volume, dims, iso, ctx=None, stream=None):
    """(blocks,) int32 CUDA tensor: exact triangles of each block at iso (iso_block_tris)."""
    import torch
    from .api import default_context
    ctx = ctx or default_context()
    nb = block_count(dims)
    out = torch.zeros(max(nb, 1), dtype=torch.int32, device=volume.device)
    g = make_grid(dims)
    check(load().iso_block_tris(ctx.handle, _ptr(volume), C.byref(g), C.c_float(iso), _ptr(out), _stream(stream)),
          ctx.handle)
    return out[:nb]


def init_params(seed=0):
    """He-initialised parameters (flat float32, the kernels' layout)."""
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, math.sqrt(2.0 / N_IN), N_IN * N_HID), np.zeros(N_HID),
             rng.normal(0, math.sqrt(2.0 / N_HID), N_HID * N_HID), np.zeros(N_HID),
             rng.normal(0, math.sqrt(1.0 / N_HID), N_HID), np.zeros(1)]
    return np.concatenate(parts).astype(np.float32)


def mlp_forward(params, stats, isos, stream=None):
    """Network output (triangles / LABEL_SCALE) for each row of stats at isos (per row)."""
    import torch
    n = stats.shape[0]
    y = torch.empty(max(n, 1), dtype=torch.float32, device=stats.device)
    if n:
        check(load().iso_mlp_forward(_ptr(params), _ptr(stats), _ptr(isos), n, _ptr(y), _stream(stream)))
    return y[:n]


def mlp_gradient(params, stats, isos, target, grads=None, loss=None, stream=None):
    """(grads, loss tensor) of the mean squared error over the rows (iso_mlp_gradient)."""
    import torch
    grads = grads if grads is not None else torch.empty(N_PARAMS, dtype=torch.float32, device=stats.device)
    loss = loss if loss is not None else torch.empty(1, dtype=torch.float32, device=stats.device)
    check(load().iso_mlp_gradient(_ptr(params), _ptr(stats), _ptr(isos), _ptr(target), stats.shape[0], _ptr(grads),
                                  _ptr(loss), _stream(stream)))
    return grads, loss


def train(stats, isos, target, epochs=6, batch=16384, lr=2e-3, seed=0, log=None):
    """Adam on (stats rows, isovalues, triangles / LABEL_SCALE) CUDA tensors; returns the parameters."""
    import torch
    lib = load()
    dev = stats.device
    params = torch.from_numpy(init_params(seed)).to(dev)
    params[-1] = float(target.mean())  # output bias at the mean label
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    grads = torch.empty_like(params)
    loss = torch.empty(1, dtype=torch.float32, device=dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    n = stats.shape[0]
    step = 0
    s = _stream(None)
    for ep in range(epochs):
        perm = torch.randperm(n, device=dev, generator=gen)
        rate = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))  # cosine decay per epoch
        total = 0.0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            xs, xi, xt = stats[idx].contiguous(), isos[idx].contiguous(), target[idx].contiguous()
            mlp_gradient(params, xs, xi, xt, grads, loss)
            step += 1
            check(lib.iso_mlp_adam(_ptr(params), _ptr(m), _ptr(v), _ptr(grads), step, C.c_float(rate), s))
            total += float(loss) * idx.numel() if log else 0.0
        if log:
            log("epoch %d loss %.5f" % (ep, total / n))
    return params


class Predictor:
    """Mesh capacities from the network: triangles = the sum over the active
    blocks of LABEL_SCALE * max(y, 0), times `margin_t`; vertices = `v_per_t` x that.  The
    margins come from the training pairs (a quantile of the exact / predicted
    ratios), so that most requests fit at the first try."""

    def __init__(self, params, margin_t=1.10, v_per_t=0.55, slack=64):
        self.params = params
        self.margin_t = margin_t
        self.v_per_t = v_per_t
        self.slack = slack

    def predict(self, items, stream=None):
        """Predicted triangles of each (stats, iso): one iso_mlp_predict launch
        (per 128 items) on `stream` (a CUDA stream handle; default: the current
        stream) and one copy of the totals back."""
        import torch
        if not items:
            return []
        sets = (_lib.IsoBlockSet * len(items))()
        for q, (st, iso) in enumerate(items):
            sets[q].stats, sets[q].n_blocks, sets[q].isoval = _ptr(st), st.shape[0], float(iso)
        totals = torch.empty(len(items), dtype=torch.float32, device=self.params.device)
        strm = torch.cuda.ExternalStream(stream) if stream is not None else \
            torch.cuda.current_stream(self.params.device)
        check(load().iso_mlp_predict(_ptr(self.params), len(items), sets, _ptr(totals), C.c_void_p(strm.cuda_stream)))
        with torch.cuda.stream(strm):
            host = totals.cpu()  # copied on strm, which it waits for
        return [float(t) * LABEL_SCALE for t in host.tolist()]

    def capacities(self, items, stream=None):
        """(cap_points, cap_tris) of each (stats, iso)."""
        return [self.capacity(t) for t in self.predict(items, stream)]

    def capacity(self, predicted_tris):
        """(cap_points, cap_tris) for a predicted triangle count: triangles times
        margin_t plus slack, vertices v_per_t times that plus slack."""
        ct = int(math.ceil(max(predicted_tris, 0.0) * self.margin_t)) + self.slack
        return int(math.ceil(ct * self.v_per_t)) + self.slack, ct

    def save(self, path=WEIGHTS):
        head = np.array([self.margin_t, self.v_per_t, self.slack], dtype=np.float32)
        np.concatenate([head, self.params.cpu().numpy()]).astype(np.float32).tofile(str(path))

    @staticmethod
    def load(path=WEIGHTS, device="cuda"):
        import torch
        a = np.fromfile(str(path), dtype=np.float32)
        if a.size != 3 + N_PARAMS:
            raise ValueError("%s: expected %d floats, found %d" % (path, 3 + N_PARAMS, a.size))
        return Predictor(torch.from_numpy(a[3:].copy()).to(device), float(a[0]), float(a[1]), int(a[2]))


def make_volume(rng, v, seed):
    dims = tuple(int(d) for d in rng.integers(32, 321, size=3))
    vol = generate_blobs(dims, 8, seed=seed) if v % 2 == 0 else generate_value_noise(dims, 4, 64, seed=seed)
    return dims, vol


def dataset(n_volumes, isos_per_volume, seed, device, ctx=None):
    """Training / evaluation pairs: per pair the active blocks' stats rows, isovalues and labels
    (exact triangles / LABEL_SCALE), plus per pair the exact (V, T) and the volume's stats."""
    import torch
    from .api import Request
    ctx = ctx or Context(device.index or 0)
    rng = np.random.default_rng(seed)
    xs, xi, xt, pairs = [], [], [], []
    for v in range(n_volumes):
        dims, vol = make_volume(rng, v, seed * 100003 + v)
        lo, hi = np.percentile(vol[:: max(1, vol.shape[0] // 16)], [5, 95])
        dv = torch.from_numpy(np.ascontiguousarray(vol).reshape(-1)).to(device)
        st = block_stats(dv, dims)
        isos = [float(np.float32(x)) for x in rng.uniform(lo, hi, isos_per_volume)]
        reqs = (_lib.IsoRequest * len(isos))(*[Request(dv, dims, iso).descriptor() for iso in isos])
        nv, nt = (C.c_int64 * len(isos))(), (C.c_int64 * len(isos))()
        check(load().iso_count_batch(ctx.handle, len(isos), reqs, nv, nt, None, _stream(None)), ctx.handle)
        for q, iso in enumerate(isos):
            tris = block_tris(dv, dims, iso, ctx)
            act = (st[:, 0] < iso) & (st[:, 1] >= iso)
            xs.append(st[act])
            xi.append(torch.full((int(act.sum()),), iso, dtype=torch.float32, device=device))
            xt.append(tris[act].float() / LABEL_SCALE)
            pairs.append({"volume": v, "dims": dims, "iso": iso, "V": nv[q], "T": nt[q], "stats": st})
        del dv
    return torch.cat(xs).contiguous(), torch.cat(xi).contiguous(), torch.cat(xt).contiguous(), pairs


def evaluate(pred, pairs):
    """Relative count error, over-allocation factor and fallback rate over (volume, isovalue) pairs."""
    t_pred = pred.predict([(p["stats"], p["iso"]) for p in pairs])
    caps = pred.capacities([(p["stats"], p["iso"]) for p in pairs])
    rel = np.array([abs(tp - p["T"]) / max(p["T"], 1) for tp, p in zip(t_pred, pairs)])
    fits = np.array([p["V"] <= cv and p["T"] <= ct for (cv, ct), p in zip(caps, pairs)])
    over = np.array([(24 * cv + 12 * ct) / max(24 * p["V"] + 12 * p["T"], 1) for (cv, ct), p in zip(caps, pairs)])
    return {"pairs": len(pairs), "rel_count_error_median": float(np.median(rel)),
            "rel_count_error_p95": float(np.percentile(rel, 95)), "rel_count_error_mean": float(rel.mean()),
            "overallocation_factor_mean": float(over[fits].mean()) if fits.any() else None,
            "fallback_rate": float(1.0 - fits.mean())}


def fit_margins(pred, pairs, q=95):
    """margin_t and v_per_t at the q-th percentile of the training pairs' exact / predicted ratios."""
    t_pred = pred.predict([(p["stats"], p["iso"]) for p in pairs])
    ratios = [p["T"] / tp for tp, p in zip(t_pred, pairs) if tp > 0 and p["T"] > 0]
    vt = [p["V"] / p["T"] for p in pairs if p["T"] > 0]
    pred.margin_t = float(np.percentile(ratios, q))
    pred.v_per_t = float(np.percentile(vt, 99.5))
    return pred


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser(description="Train and evaluate the output-size network.")
    ap.add_argument("--volumes", type=int, default=500)
    ap.add_argument("--isos", type=int, default=40)
    ap.add_argument("--eval-volumes", type=int, default=50)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--out", default=str(WEIGHTS))
    args = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    t0 = time.time()
    xs, xi, xt, train_pairs = dataset(args.volumes, args.isos, seed=1, device=dev)
    t1 = time.time()
    params = train(xs, xi, xt, epochs=args.epochs, log=lambda s: print(s, flush=True))
    torch.cuda.synchronize()
    t2 = time.time()
    pred = fit_margins(Predictor(params), train_pairs)
    _, _, _, eval_pairs = dataset(args.eval_volumes, args.isos, seed=2, device=dev)
    # without the network: active blocks x the training set's mean triangles per active block
    mean_per_block = float(xt.mean()) * LABEL_SCALE
    base = [(p["stats"], p["iso"]) for p in eval_pairs]
    base_t = [float(((st[:, 0] < iso) & (st[:, 1] >= iso)).sum()) * mean_per_block for st, iso in base]
    base_rel = np.array([abs(b - p["T"]) / max(p["T"], 1) for b, p in zip(base_t, eval_pairs)])
    report = {"train_pairs": len(train_pairs), "train_blocks": int(xs.shape[0]), "eval_pairs": len(eval_pairs),
              "data_seconds": t1 - t0, "train_seconds": t2 - t1, "margin_t": pred.margin_t, "v_per_t": pred.v_per_t,
              "train": evaluate(pred, train_pairs), "held_out": evaluate(pred, eval_pairs),
              "held_out_without_network": {"estimator": "active blocks x mean triangles per active block",
                                           "rel_count_error_median": float(np.median(base_rel)),
                                           "rel_count_error_p95": float(np.percentile(base_rel, 95))}}
    pred.save(args.out)
    print(json.dumps(report), flush=True)


if __name__ == "__main__":
    main()
