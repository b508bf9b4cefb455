"""Gradient descent on a scene's material albedos, with checkpoints.

The adjoint trace (tracer_trace_adjoint) gives dLoss/d(albedo) for an image
loss; this module turns those gradients into parameter updates (Adam, then a
clamp to the valid albedo range) and saves / restores the whole optimisation
state as an .npz file, so that a long run (the 1024^2 x 64 spp, 1M-triangle
gradient descent) can stop and resume with bit-identical parameters.

No counterpart in the reference, which renders with fixed materials.
"""
from __future__ import annotations

import os

import numpy as np


class AlbedoDescent:
    """Adam (Kingma & Ba 2015: first/second moment estimates with bias
    correction) on an (n_materials, 3) albedo table, clamped to [lo, hi] after
    every step.  State in float64; `albedo` gives the float32 table to upload."""

    def __init__(self, start: np.ndarray, lr: float = 0.01, beta1: float = 0.9, beta2: float = 0.999,
                 eps: float = 1e-8, lo: float = 1e-3, hi: float = 1.0):
        self.x = np.array(start, np.float64).reshape(-1, 3)
        self.m = np.zeros_like(self.x)
        self.v = np.zeros_like(self.x)
        self.t = 0
        self.hp = dict(lr=float(lr), beta1=float(beta1), beta2=float(beta2), eps=float(eps), lo=float(lo),
                       hi=float(hi))
        self.seen = np.zeros(len(self.x), bool)  # materials that ever received a gradient
        self.log: dict[str, list] = {}

    @property
    def albedo(self) -> np.ndarray:
        return self.x.astype(np.float32)

    def step(self, grad: np.ndarray) -> None:
        g = np.asarray(grad, np.float64).reshape(self.x.shape)
        h = self.hp
        self.t += 1
        self.m = h["beta1"] * self.m + (1.0 - h["beta1"]) * g
        self.v = h["beta2"] * self.v + (1.0 - h["beta2"]) * g * g
        mhat = self.m / (1.0 - h["beta1"] ** self.t)
        vhat = self.v / (1.0 - h["beta2"] ** self.t)
        self.x = np.clip(self.x - h["lr"] * mhat / (np.sqrt(vhat) + h["eps"]), h["lo"], h["hi"])
        self.seen |= (g != 0).any(axis=1)

    def record(self, **values) -> None:
        """Per-step measurements kept with the state (saved in checkpoints)."""
        for k, v in values.items():
            self.log.setdefault(k, []).append(float(v))

    def save(self, path: str) -> None:
        """Writes the state atomically (a temporary file, then a rename)."""
        tmp = path + ".tmp.npz"
        np.savez(tmp, x=self.x, m=self.m, v=self.v, t=np.int64(self.t), seen=self.seen,
                 hp_keys=np.array(list(self.hp)), hp_vals=np.array(list(self.hp.values())),
                 log_keys=np.array(list(self.log), dtype=str),
                 **{f"log_{k}": np.array(v, np.float64) for k, v in self.log.items()})
        os.replace(tmp, path)

    @classmethod
    def load(cls, path: str) -> "AlbedoDescent":
        with np.load(path, allow_pickle=False) as z:
            hp = {str(k): float(v) for k, v in zip(z["hp_keys"], z["hp_vals"])}
            d = cls(z["x"], **hp)
            d.m, d.v, d.t, d.seen = z["m"].copy(), z["v"].copy(), int(z["t"]), z["seen"].copy()
            d.log = {str(k): z[f"log_{k}"].tolist() for k in z["log_keys"]}
        return d
