"""Batched ensembles: many independent PBSM3D domains (meshes of any sizes,
each with its own perturbed constants) advanced together by one context.

The library solves the disjoint union of the members' systems as one joint
system, with each member's own "suspension/deposition present" test and its
own relative tolerance (include/pbsm3d.h, pbsm3d_ensemble_create).  The
reference runs one domain per process; an ensemble there is N separate runs
of PBSM3D (src/modules/PBSM3D.cpp), which is what each member reproduces.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .pbsm3d import FORCING_KEYS, OUTPUT_KEYS, PBSM3D, ModuleError


@dataclass
class MemberParams:
    ustar_th_scale: float = 1.0   # multiplies the threshold friction velocity
    z0_snow: float = 0.01         # aerodynamic roughness of snow (m)
    settling_scale: float = 1.0   # multiplies the settling velocity


def perturbed_members(n: int, seed: int) -> list[MemberParams]:
    """Threshold friction velocity +-20 %, roughness log-uniform in
    [1e-4, 1e-2] m, settling-velocity scale +-15 %."""
    r = np.random.default_rng(seed)
    return [MemberParams(float(r.uniform(0.8, 1.2)), float(10.0 ** r.uniform(-4.0, -2.0)),
                         float(r.uniform(0.85, 1.15))) for _ in range(n)]


class Ensemble(PBSM3D):
    """PBSM3D over several member domains in one context.  ``run`` takes and
    returns the members' arrays concatenated in member order; ``run_members``
    takes a list of per-member forcings and returns per-member outputs."""

    def __init__(self, cfg: dict):
        super().__init__(cfg)
        self.offsets = None

    def init(self, meshes, members, **solver):
        if len(meshes) != len(members) or not meshes:
            raise ModuleError("an ensemble needs one parameter set per mesh")
        lib = capi.load()
        cfg = self.make_config(lib, **solver)
        n = len(meshes)
        descs = (capi.MeshDesc * n)(*[capi.mesh_desc(m, self._keep) for m in meshes])
        mem = (capi.Member * n)(*[capi.Member(p.ustar_th_scale, p.z0_snow, p.settling_scale) for p in members])
        ctx = C.c_void_p()
        rc = lib.pbsm3d_ensemble_create(n, descs, mem, C.byref(cfg), C.byref(ctx))
        if rc != 0:
            raise ModuleError(f"pbsm3d_ensemble_create: {capi.STATUS_NAMES.get(rc, rc)}: "
                              f"{lib.pbsm3d_last_error(None).decode()}")
        self._lib = lib
        self._ctx = ctx
        off = np.empty(n + 1, np.int64)
        got = lib.pbsm3d_member_offsets(ctx, off.ctypes.data_as(C.POINTER(C.c_int64)))
        if got != n:
            raise ModuleError("pbsm3d_member_offsets disagrees with the member count")
        self.offsets = off
        self.n_faces = int(off[-1])
        self.n_members = n

    def concat_forcing(self, forcings) -> dict:
        src = [f if isinstance(f, dict) else f.arrays() for f in forcings]
        out = {}
        for k in FORCING_KEYS:
            have = [s.get(k) is not None for s in src]
            if not any(have):
                continue
            if not all(have):
                raise ModuleError(f"forcing {k} given for some members only")
            out[k] = np.concatenate([np.asarray(s[k], np.float64) for s in src])
        return out

    def split(self, out: dict) -> list[dict]:
        o, L, T = self.offsets, self.nLayer, self.n_faces
        res = []
        for m in range(self.n_members):
            d = {k: out[k][o[m]:o[m + 1]] for k in OUTPUT_KEYS if k in out}
            if "c" in out:
                d["c"] = out["c"].reshape(L, T)[:, o[m]:o[m + 1]].ravel()
            res.append(d)
        return res

    def run_members(self, forcings, dt: float, want_c: bool = False) -> list[dict]:
        if len(forcings) != self.n_members:
            raise ModuleError("one forcing per member")
        return self.split(self.run(self.concat_forcing(forcings), dt, want_c=want_c))
