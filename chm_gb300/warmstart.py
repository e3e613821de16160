"""Learned warm start of the suspension solve: training data from plain-solver
solutions, GPU training with the library's tensor-core kernels, and the
packed parameter file.

Parameters are one FP32 vector (include/pbsm3d.h, pbsm3d_set_mlp):
W0[128][14] b0[128] W1[128][128] b1[128] W2[128][128] b2[128] w3[128] b3.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import capi, synth
from .pbsm3d import PBSM3D, ModuleError

NUM_FEAT = 14
HID = 128
SHAPES = [("W0", (HID, NUM_FEAT)), ("b0", (HID,)), ("W1", (HID, HID)), ("b1", (HID,)), ("W2", (HID, HID)),
          ("b2", (HID,)), ("w3", (HID,)), ("b3", (1,))]
WEIGHTS_FILE = Path(__file__).resolve().parent / "data" / "warmstart_mlp.npz"


def n_params() -> int:
    return sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.asarray(d[name], np.float32).ravel() for name, _ in SHAPES]).astype(np.float32)


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised weights, zero biases."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            d[name] = rng.normal(0, np.sqrt(2.0 / shape[1]), shape)
        elif name == "w3":
            d[name] = rng.normal(0, np.sqrt(1.0 / HID), shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def collect(seeds, n_points: int, side: float, nLayer: int, steps: int, rows_per_step: int, wind: float = 8.0,
            rng_seed: int = 0, workloads=None):
    """(features, targets) as CUDA tensors: `rows_per_step` random rows of
    every step of plain FP64 solves on the seeded meshes (c_prev of the first
    step is zero, as in a cold start).  `workloads`, when given, are the
    seeds' prebuilt workloads (in seed order)."""
    import torch
    lib = capi.load()
    rng = np.random.default_rng(rng_seed)
    feats, targs = [], []
    for k, seed in enumerate(seeds):
        w = workloads[k] if workloads is not None else synth.Workload(n_points, side, seed=seed, wind_scale=wind)
        m = PBSM3D({"nLayer": str(nLayer)})
        m.init(w.mesh)
        rows = w.mesh.n_faces * nLayer
        f_dev = torch.empty((rows, NUM_FEAT), dtype=torch.float32, device="cuda")
        t_dev = torch.empty(rows, dtype=torch.float32, device="cuda")
        for s in range(steps):
            out = m.run(w.forcing(s), 3600.0)
            if not m.last_stats["suspension_present"]:
                w.apply_drift(out["drift_mass"])
                continue
            rc = lib.pbsm3d_mlp_features(m._ctx, _ptr(f_dev), _ptr(t_dev), 1)
            if rc != 0:
                raise ModuleError(lib.pbsm3d_last_error(m._ctx).decode())
            pick = torch.from_numpy(rng.choice(rows, size=min(rows_per_step, rows), replace=False)).cuda()
            feats.append(f_dev[pick].clone())
            targs.append(t_dev[pick].clone())
            w.apply_drift(out["drift_mass"])
        m.close()
    return torch.cat(feats), torch.cat(targs)


def feature_stats(feat) -> tuple[np.ndarray, np.ndarray]:
    f = feat.double()
    mean = f.mean(0).cpu().numpy().astype(np.float32)
    std = f.std(0).cpu().numpy()
    scale = (1.0 / np.maximum(std, 1e-6)).astype(np.float32)
    return mean, scale


class Trainer:
    def __init__(self, params: np.ndarray, mean, scale, batch: int = 8192):
        self.lib = capi.load()
        self.batch = batch
        self.h = C.c_void_p()
        p = np.ascontiguousarray(params, np.float32)
        rc = self.lib.pbsm3d_mlp_trainer_create(batch, capi.ptr(p, C.c_float), capi.ptr(np.ascontiguousarray(mean),
                                                C.c_float), capi.ptr(np.ascontiguousarray(scale), C.c_float),
                                                C.byref(self.h))
        if rc != 0:
            raise ModuleError(self.lib.pbsm3d_last_error(None).decode())

    def train(self, feat, target, steps: int, lr: float, seed: int = 0) -> np.ndarray:
        losses = np.empty(steps, np.float32)
        rc = self.lib.pbsm3d_mlp_train(self.h, _ptr(feat), _ptr(target), feat.shape[0], steps, lr, seed,
                                       capi.ptr(losses, C.c_float))
        if rc != 0:
            raise ModuleError(self.lib.pbsm3d_last_error(None).decode())
        return losses

    def grad(self, feat: np.ndarray, target: np.ndarray):
        g = np.empty(n_params(), np.float32)
        loss = np.zeros(1, np.float32)
        y = np.empty(self.batch, np.float32)
        rc = self.lib.pbsm3d_mlp_grad(self.h, capi.ptr(np.ascontiguousarray(feat, np.float32), C.c_float),
                                      capi.ptr(np.ascontiguousarray(target, np.float32), C.c_float),
                                      capi.ptr(g, C.c_float), capi.ptr(loss, C.c_float), capi.ptr(y, C.c_float))
        if rc != 0:
            raise ModuleError(self.lib.pbsm3d_last_error(None).decode())
        return g, float(loss[0]), y

    def params(self) -> np.ndarray:
        p = np.empty(n_params(), np.float32)
        self.lib.pbsm3d_mlp_get_params(self.h, capi.ptr(p, C.c_float))
        return p

    def close(self):
        if self.h:
            self.lib.pbsm3d_mlp_trainer_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def save(path, params, mean, scale, **meta):
    Path(path).parent.mkdir(parents=True, exist_ok=True)
    np.savez(path, params=params, mean=mean, scale=scale, **meta)


def load(path=WEIGHTS_FILE):
    d = np.load(path)
    return d["params"].astype(np.float32), d["mean"].astype(np.float32), d["scale"].astype(np.float32)


def set_mlp(module: PBSM3D, params, mean, scale):
    lib = module._lib
    rc = lib.pbsm3d_set_mlp(module._ctx, capi.ptr(np.ascontiguousarray(params, np.float32), C.c_float),
                            capi.ptr(np.ascontiguousarray(mean, np.float32), C.c_float),
                            capi.ptr(np.ascontiguousarray(scale, np.float32), C.c_float))
    if rc != 0:
        raise ModuleError(lib.pbsm3d_last_error(module._ctx).decode())


def predict(module: PBSM3D) -> np.ndarray:
    out = np.empty(module.n_faces * module.nLayer)
    rc = module._lib.pbsm3d_mlp_predict(module._ctx, capi.ptr(out))
    if rc != 0:
        raise ModuleError(module._lib.pbsm3d_last_error(module._ctx).decode())
    return out


def features(module: PBSM3D):
    rows = module.n_faces * module.nLayer
    f = np.empty((rows, NUM_FEAT), np.float32)
    t = np.empty(rows, np.float32)
    rc = module._lib.pbsm3d_mlp_features(module._ctx, C.c_void_p(f.ctypes.data), C.c_void_p(t.ctypes.data), 0)
    if rc != 0:
        raise ModuleError(module._lib.pbsm3d_last_error(module._ctx).decode())
    return f, t


def train_from_solutions(train_seeds, n_points, side, nLayer, steps_per_seed, rows_per_step, train_steps, lr=1e-3,
                         batch=8192, seed=0, wind=8.0, workloads=None):
    """Collect plain-solver solutions on the training seeds and fit the MLP on the GPU."""
    feat, targ = collect(train_seeds, n_points, side, nLayer, steps_per_seed, rows_per_step, wind=wind,
                         rng_seed=seed, workloads=workloads)
    mean, scale = feature_stats(feat)
    tr = Trainer(init_params(seed), mean, scale, batch=batch)
    losses = tr.train(feat, targ, train_steps, lr, seed)
    params = tr.params()
    tr.close()
    return params, mean, scale, losses, int(feat.shape[0])
