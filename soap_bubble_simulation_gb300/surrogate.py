"""Drainage surrogate: a 4-layer convolutional neural operator that advances a GPUDrainageSimulator
film (drainage.wgsl:72-202, Marangoni off) by SURROGATE_STEPS = 64 passes in one forward pass.

The network, its input features and its parameter layout are fixed by include/sbs_nn.h; the
activation is GELU (the default, ``activation="gelu"``) or hard-swish (``"hswish"``). It is
trained here on trajectories of the plain GPU solver by the library's own tensor-core forward and
backward kernels, and it runs either layer by layer (``mode="layered"``) or as one fused tcgen05
kernel (``mode="fused"``). ``rollout`` lets the plain solver check every K-th interval and take
over when the masked relative L-inf error exceeds a tolerance.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import replace

import numpy as np

from . import _native as N
from .drainage import DrainageParams, GPUDrainageSimulator

SURROGATE_STEPS = N.NN_STEPS
NUM_PARAMS = N.NN_PARAMS
_MODES = {"layered": N.NN_LAYERED, "fused": N.NN_FUSED}
ACTIVATIONS = {"gelu": N.NN_ACT_GELU, "hswish": N.NN_ACT_HSWISH}


class SurrogateEval(C.Structure):
    _fields_ = [("loss", C.c_double), ("loss_identity", C.c_double), ("rel_linf", C.c_double),
                ("rel_linf_identity", C.c_double)]


class SurrogateStats(C.Structure):
    _fields_ = [("rollouts", C.c_uint32), ("surrogate", C.c_uint32), ("plain", C.c_uint32), ("checks", C.c_uint32),
                ("failed_checks", C.c_uint32), ("pad", C.c_uint32), ("max_check_error", C.c_double),
                ("last_check_error", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


def field_params(nt: int, np_: int, **kw) -> DrainageParams:
    """DrainageParams for an nt x np_ (theta x phi) grid with overrides."""
    return replace(DrainageParams(), grid_width=int(np_), grid_height=int(nt), **kw)


def _param_array(params, nf: int):
    if isinstance(params, DrainageParams):
        params = [params] * nf
    if len(params) != nf:
        raise ValueError("one DrainageParams per field")
    arr = (N.SbsDrainageParams * nf)()
    for k, p in enumerate(params):
        arr[k] = p.to_c()
    return arr


def _fields(h, c):
    h = np.ascontiguousarray(h, dtype=np.float32)
    c = np.ascontiguousarray(c, dtype=np.float32)
    if h.ndim == 2:
        h, c = h[None], c[None]
    if h.shape != c.shape or h.ndim != 3:
        raise ValueError("h and c must both be [nt][np] or [nf][nt][np]")
    return h, c


def _mode(mode: str) -> int:
    try:
        return _MODES[mode]
    except KeyError:
        raise ValueError(f"mode must be one of {sorted(_MODES)}") from None


class DrainageSurrogate:
    def __init__(self, seed: int = 0, activation: str = "gelu"):
        self._h = C.c_void_p()
        N.call("sbs_surrogate_create", C.c_uint64(seed), C.byref(self._h))
        self.activation = activation

    def close(self):
        if self._h:
            N.lib().sbs_surrogate_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ parameters
    @property
    def params(self) -> np.ndarray:
        out = np.empty(NUM_PARAMS, dtype=np.float32)
        N.call("sbs_surrogate_get_params", self._h, N.ptr(out), out.size)
        return out

    @params.setter
    def params(self, theta) -> None:
        theta = np.ascontiguousarray(theta, dtype=np.float32)
        if theta.size != NUM_PARAMS:
            raise ValueError(f"expected {NUM_PARAMS} parameters")
        N.call("sbs_surrogate_set_params", self._h, N.ptr(theta), theta.size)

    @property
    def activation(self) -> str:
        out = C.c_int()
        N.call("sbs_surrogate_get_activation", self._h, C.byref(out))
        return {v: k for k, v in ACTIVATIONS.items()}[out.value]

    @activation.setter
    def activation(self, name: str) -> None:
        """Weights trained with one activation do not fit the other: set it before training."""
        if name not in ACTIVATIONS:
            raise ValueError(f"activation must be one of {sorted(ACTIVATIONS)}")
        N.call("sbs_surrogate_set_activation", self._h, ACTIVATIONS[name])

    # ------------------------------------------------------------------ network
    def features(self, h, c, params) -> np.ndarray:
        h, c = _fields(h, c)
        nf = h.shape[0]
        x = np.empty(h.shape + (16,), dtype=np.float32)
        N.call("sbs_surrogate_features", self._h, nf, N.ptr(h), N.ptr(c), _param_array(params, nf), N.ptr(x),
               N.MEM_HOST)
        return x

    def forward(self, h, c, params, mode: str = "layered") -> np.ndarray:
        h, c = _fields(h, c)
        nf = h.shape[0]
        y = np.empty(h.shape, dtype=np.float32)
        N.call("sbs_surrogate_forward", self._h, nf, N.ptr(h), N.ptr(c), _param_array(params, nf), N.ptr(y),
               _mode(mode), N.MEM_HOST)
        return y

    def loss_grad(self, h, c, params, target):
        h, c = _fields(h, c)
        nf = h.shape[0]
        t = np.ascontiguousarray(target, dtype=np.float32).reshape(h.shape)
        g = np.empty(NUM_PARAMS, dtype=np.float32)
        loss = C.c_double()
        N.call("sbs_surrogate_loss_grad", self._h, nf, N.ptr(h), N.ptr(c), _param_array(params, nf), N.ptr(t),
               C.byref(loss), N.ptr(g))
        return loss.value, g

    # ------------------------------------------------------------------ training
    def add_trajectory(self, h0, c0, params: DrainageParams, pairs: int = 4, substeps: int = 0) -> None:
        h0 = np.ascontiguousarray(h0, dtype=np.float32)
        c0 = np.ascontiguousarray(c0, dtype=np.float32)
        if h0.shape != (params.grid_height, params.grid_width) or c0.shape != h0.shape:
            raise ValueError("h0 / c0 must be grid_height x grid_width")
        p = params.to_c()
        N.call("sbs_surrogate_add_trajectory", self._h, N.ptr(h0), N.ptr(c0), C.byref(p), int(pairs), int(substeps))

    def num_trajectories(self) -> int:
        out = C.c_uint32()
        N.call("sbs_surrogate_num_trajectories", self._h, C.byref(out))
        return out.value

    def clear_data(self) -> None:
        N.call("sbs_surrogate_clear_data", self._h)

    def train(self, n_train: int, iters: int, batch: int = 4, lr: float = 2e-3, seed: int = 0) -> np.ndarray:
        losses = np.empty(int(iters), dtype=np.float32)
        N.call("sbs_surrogate_train", self._h, int(n_train), int(iters), int(batch), float(lr), C.c_uint64(seed),
               N.ptr(losses))
        return losses

    def evaluate(self, first: int, count: int, mode: str = "layered") -> dict:
        e = SurrogateEval()
        N.call("sbs_surrogate_evaluate", self._h, int(first), int(count), _mode(mode), C.byref(e))
        return {k: getattr(e, k) for k, _ in e._fields_}

    # ------------------------------------------------------------------ rollout
    def advance(self, sim: GPUDrainageSimulator, mode: str = "fused") -> None:
        N.call("sbs_surrogate_advance", self._h, sim._h, _mode(mode))

    def rollout(self, sim: GPUDrainageSimulator, passes: int, check_every: int = 8, tol: float = 1e-3,
                mode: str = "fused") -> dict:
        st = SurrogateStats()
        N.call("sbs_surrogate_rollout", self._h, sim._h, int(passes), int(check_every), float(tol), _mode(mode),
               C.byref(st))
        return st.as_dict()

    def stream(self) -> int:
        out = C.c_void_p()
        N.call("sbs_surrogate_stream", self._h, C.byref(out))
        return out.value or 0


def masked_error(a, b) -> float:
    """max |a - b| / max |b| over rows with sin(theta) >= 0.2 (rows 1..nt-2) of two nt x np fields."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    if a.shape != b.shape or a.ndim != 2:
        raise ValueError("two nt x np fields expected")
    out = C.c_double()
    N.call("sbs_surrogate_masked_error", N.ptr(a), N.ptr(b), a.shape[0], a.shape[1], N.MEM_HOST, C.byref(out))
    return out.value
