"""Training and evaluation of the learned pressure warm start.

The network (fl_unet_*, see include/flowlab_gb300.h) predicts a correction
of the previous step's pressure from (b / s_b, fluid mask, p_prev / s_p).
Training pairs come from the engine itself: each step of a running scene
gives the step's right-hand side b, the warm start p_prev it started from
and the converged pressure p_conv the multigrid reached, and the target is
(p_conv - p_prev) / s_p on fluid cells. Scenes: the thermal plume, the
turbulence grid and seeded batched-scene members at every training size
(256^2, 512^2 and 1024^2 by default), each restarted (new seed) after a
fixed number of steps; a training step takes one size, as many pairs as
fill its pixel budget (16 at 256^2, 4 at 512^2, 1 at 1024^2), the sizes
in turn.

  python -m flowlab_gb300.warmstart train --pairs 20000 --out weights.npz
  python -m flowlab_gb300.warmstart evaluate --weights weights.npz

Evaluation runs the same scene twice, plain multigrid and warm-started
multigrid, both to the same tolerance, and reports V-cycles per step and
steps/s (CUDA events on the engine's stream).
"""
import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

from . import configs, native
from .native import f32, ptr

FLUID = 0
HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "weights", "warmstart_unet.npz")


def features(b, label, p_prev):
    """The network input and the scales, as the engine computes them on the
    device: s_b = RMS of b over fluid cells, s_p = RMS of p_prev over fluid
    cells (s_b when p_prev vanishes); x = (b / s_b, mask, p_prev / s_p)."""
    fl = label == FLUID
    b = np.asarray(b, np.float32)
    p = np.asarray(p_prev, np.float32)
    n = max(1, int(fl.sum()))
    sb = float(np.sqrt(np.sum(b[fl].astype(np.float64) ** 2) / n))
    sp = float(np.sqrt(np.sum(p[fl].astype(np.float64) ** 2) / n))
    if not sp > 0:
        sp = sb
    ib = np.float32(1.0 / sb) if sb > 0 else np.float32(0)
    ip = np.float32(1.0 / sp) if sp > 0 else np.float32(0)
    x = np.zeros(b.shape + (3,), np.float32)
    x[..., 0] = np.where(fl, b * ib, 0)
    x[..., 1] = fl
    x[..., 2] = np.where(fl, p * ip, 0)
    return x, sb, sp


class PairSource:
    """One running scene on the engine; each step yields a training pair."""

    def __init__(self, kind, size, seed, restart_every=150, skip=2):
        self.kind, self.size, self.seed, self.restart_every, self.skip = kind, size, seed, restart_every, skip
        self.eng = None
        self._reset()

    def _reset(self):
        if self.eng is not None:
            self.eng.close()
        n = self.size
        if self.kind == "plume":
            g, f, patch = configs.plume(n)
            prm = configs.plume_params(tol=1e-6, max_cycles=30, mixed=1)
        elif self.kind == "turbulence":
            g, f, patch = configs.turbulence(n)
            prm = configs.turbulence_params(tol=1e-6, max_cycles=40)
        else:
            g, f, patch = configs.random_scene(n, self.seed)
            prm = configs.random_scene_params(tol=1e-6, mixed=1, max_cycles=30)
        self.seed += 1000
        self.eng = native.Engine(g.nx, g.ny, g.h, params=prm)
        if patch is not None:
            self.eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        self.eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)),
                      ptr(f.label), ptr(f32(f.dye)))
        self.label = f.label.reshape(n, n).copy()
        self.steps = 0
        self.p = np.zeros((n, n), np.float32)
        self.b = np.zeros((n, n), np.float32)

    def pair(self):
        """The next step's (x, target, mask). The first steps after a reset
        (p_prev = 0, the cold start no warm start sees in a running scene)
        are stepped but not returned."""
        if self.steps >= self.restart_every:
            self._reset()
        while self.steps < self.skip:
            self.eng.call("fl_step_auto", 1, None)
            self.steps += 1
        e = self.eng
        e.call("fl_read_pressure", native.FL_F32, ptr(self.p))
        p_prev = self.p.copy()
        e.call("fl_step_auto", 1, None)
        e.call("fl_read_rhs", native.FL_F32, ptr(self.b))
        e.call("fl_read_pressure", native.FL_F32, ptr(self.p))
        self.steps += 1
        x, sb, sp = features(self.b, self.label, p_prev)
        fl = (self.label == FLUID)
        t = np.where(fl, (self.p - p_prev) / np.float32(sp if sp > 0 else 1), 0).astype(np.float32)
        return x, t, fl.astype(np.float32)

    def close(self):
        if self.eng is not None:
            self.eng.close()
            self.eng = None


LAYERS = [(3, 32, 3, 0), (32, 32, 3, 0), (32, 64, 3, 1), (64, 64, 3, 1), (64, 96, 3, 2), (96, 96, 3, 2),
          (96, 128, 3, 3), (128, 128, 3, 3), (224, 96, 3, 2), (96, 96, 3, 2), (160, 64, 3, 1), (64, 64, 3, 1),
          (96, 32, 3, 0), (32, 32, 3, 0), (32, 1, 1, 0)]  # (cin, cout, k, level)


def forward_flops(h, w):
    """Multiply-add FLOPs (2 per MAC) of one forward pass on an h x w grid;
    and the part the tensor cores run (3x3 convolutions with >= 32 inputs)."""
    total = tc = 0
    for cin, cout, k, lev in LAYERS:
        f = 2.0 * k * k * cin * cout * (h >> lev) * (w >> lev)
        total += f
        if k == 3 and cin % 32 == 0:
            tc += f
    return total, tc


def he_init(seed=0):
    """He-normal weights, zero biases, zero head: the untrained network
    returns p_prev unchanged. Same layout as fl_unet_set_params."""
    rng = np.random.default_rng(seed)
    layers = [(3, 32, 3), (32, 32, 3), (32, 64, 3), (64, 64, 3), (64, 96, 3), (96, 96, 3), (96, 128, 3),
              (128, 128, 3), (224, 96, 3), (96, 96, 3), (160, 64, 3), (64, 64, 3), (96, 32, 3), (32, 32, 3),
              (32, 1, 1)]
    chunks = []
    for li, (cin, cout, k) in enumerate(layers):
        nw = cout * k * k * cin
        w = np.zeros(nw, np.float32) if li == len(layers) - 1 else \
            (rng.standard_normal(nw) * np.sqrt(2.0 / (k * k * cin))).astype(np.float32)
        chunks += [w, np.zeros(cout, np.float32)]
    return np.concatenate(chunks)


def train(pairs=20000, sizes=(256, 512, 1024), pixels=1 << 20, lr=1e-3, seed=0, log=None, params=None):
    """Trains a fresh network (or `params`) on `pairs` pairs generated while
    training, each used once. Training steps take the sizes in turn, each
    with a batch of pixels // size^2 pairs of that size (at least one), the
    pairs drawn in turn from that size's plume, turbulence-grid and two
    batched-scene sources. Returns (network, per-step losses)."""
    net = native.Unet(max(pixels, max(sizes) ** 2))
    net.set_params(he_init(seed) if params is None else params)
    kinds = ["plume", "turbulence", "random", "random"]
    sources = {n: [PairSource(k, n, seed + 17 * i + 1000003 * j) for i, k in enumerate(kinds)]
               for j, n in enumerate(sizes)}
    turn = {n: 0 for n in sizes}
    losses = []
    t0 = time.time()
    done = s = 0
    try:
        while done < pairs:
            n = sizes[s % len(sizes)]
            batch = min(max(1, pixels // (n * n)), pairs - done)
            xs, ts, ms = [], [], []
            for _ in range(batch):
                src = sources[n][turn[n] % len(kinds)]
                turn[n] += 1
                x, t, m = src.pair()
                xs.append(x)
                ts.append(t)
                ms.append(m)
            loss = net.train_step(np.stack(xs), np.stack(ts), np.stack(ms), lr=lr)
            losses.append(loss)
            done += batch
            s += 1
            if log and s % 100 == 0:
                log("step %d, %d/%d pairs, loss %.4g (%.0f s)" % (s, done, pairs, float(np.mean(losses[-100:])),
                                                                   time.time() - t0))
    finally:
        for srcs in sources.values():
            for src in srcs:
                src.close()
    return net, losses


def run_scene(n, steps, warmup, net=None, workload="plume"):
    """Steps a scene, with or without the warm start; returns the per-step
    V-cycles, relative residuals and device milliseconds."""
    import torch

    if workload == "plume":
        g, f, patch = configs.plume(n)
        prm = configs.plume_params()
    else:
        g, f, patch = configs.turbulence(n)
        prm = configs.turbulence_params()
    eng = native.Engine(g.nx, g.ny, g.h, params=prm)
    try:
        if patch is not None:
            eng.call("fl_set_dye_patch", patch.i0, patch.j0, patch.nx, patch.ny, ptr(f32(patch.data)))
        eng.call("fl_upload_fields", native.FL_F32, ptr(f32(f.u)), ptr(f32(f.v)), ptr(f32(f.p)), ptr(f.label),
                 ptr(f32(f.dye)))
        if net is not None:
            eng.call("fl_set_warm_start", net.h)
        for _ in range(warmup):
            eng.call("fl_step_auto", 1, None)
        eng.call("fl_synchronize")
        stream = torch.cuda.ExternalStream(eng.stream())
        cyc, rr, ms = [], [], []
        for _ in range(steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.call("fl_step_auto", 1, None)
            b.record(stream)
            st = eng.stats()
            cyc.append(st["cycles"])
            rr.append(st["rel_residual"])
            ms.append(a.elapsed_time(b))
    finally:
        eng.close()
    return cyc, rr, ms


def evaluate(params, n=1024, steps=30, warmup=10, workload="plume"):
    net = native.Unet(n * n)
    try:
        net.set_params(params)
        pc, pr, pm = run_scene(n, steps, warmup, None, workload)
        cc, cr, cm = run_scene(n, steps, warmup, net, workload)
    finally:
        net.close()
    return {
        "grid": [n, n], "workload": workload, "steps": steps, "warmup": warmup,
        "plain": {"vcycles_per_step": float(np.mean(pc)), "steps_per_s": 1000.0 / float(np.mean(pm)),
                  "rel_residual_max": float(np.max(pr))},
        "cnn": {"vcycles_per_step": float(np.mean(cc)), "steps_per_s": 1000.0 / float(np.mean(cm)),
                "rel_residual_max": float(np.max(cr))},
        "vcycles_saved_per_step": float(np.mean(pc) - np.mean(cc)),
    }


def save(path, params, meta):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params=np.asarray(params, np.float32), meta=json.dumps(meta))


def time_forward(params, size, batch=1, repeat=3, seed=0):
    """fl_unet_forward on a seeded standard-normal input of batch x size x
    size x 3: wall-clock ms per call (host input and output copies
    included), after one untimed call."""
    x = np.random.default_rng(seed).standard_normal((batch, size, size, 3)).astype(np.float32)
    net = native.Unet(batch * size * size)
    try:
        net.set_params(params)
        net.forward(x)
        t0 = time.perf_counter()
        for _ in range(repeat):
            out = net.forward(x)
        ms = 1000.0 * (time.perf_counter() - t0) / max(1, repeat)
    finally:
        net.close()
    flops, _ = forward_flops(size, size)
    return {"size": size, "batch": batch, "ms_per_call": ms, "out_mean_abs": float(np.abs(out).mean()),
            "forward_flops": flops * batch}


def load(path):
    z = np.load(path)
    return z["params"], json.loads(str(z["meta"]))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=20000)
    t.add_argument("--sizes", default="256,512,1024", help="training grid sides, taken in turn")
    t.add_argument("--pixels", type=int, default=1 << 20, help="pixels per training step (batch = pixels // side^2)")
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--out", default=DEFAULT_WEIGHTS)
    t.add_argument("--eval-size", type=int, default=1024)
    e = sub.add_parser("evaluate")
    e.add_argument("--weights", default=DEFAULT_WEIGHTS)
    e.add_argument("--size", type=int, default=1024)
    e.add_argument("--steps", type=int, default=30)
    f = sub.add_parser("forward", help="time the forward pass on a seeded random input")
    f.add_argument("--weights", default=DEFAULT_WEIGHTS)
    f.add_argument("--size", type=int, default=1024)
    f.add_argument("--batch", type=int, default=1)
    f.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args(argv)
    from . import build

    build.build()
    if a.cmd == "train":
        t0 = time.time()
        sizes = tuple(int(x) for x in a.sizes.split(","))
        net, losses = train(a.pairs, sizes, a.pixels, a.lr, a.seed, log=lambda m: print(m, flush=True))
        params = net.get_params()
        net.close()
        meta = {"pairs": a.pairs, "sizes": list(sizes), "pixels_per_step": a.pixels, "lr": a.lr, "seed": a.seed,
                "train_seconds": time.time() - t0, "loss_first100": float(np.mean(losses[:100])),
                "loss_last100": float(np.mean(losses[-100:]))}
        if a.eval_size:
            meta["evaluation"] = evaluate(params, a.eval_size)
        save(a.out, params, meta)
        print(json.dumps(meta), flush=True)
    elif a.cmd == "forward":
        params, _ = load(a.weights)
        print(json.dumps(time_forward(params, a.size, a.batch, a.repeat)), flush=True)
    else:
        params, meta = load(a.weights)
        print(json.dumps(evaluate(params, a.size, a.steps)), flush=True)


if __name__ == "__main__":
    sys.exit(main())
