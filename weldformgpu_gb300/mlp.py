"""The learned warm start of the Johnson-Cook return map.

A 4 -> 64 -> 64 -> 1 SiLU network proposes dlambda / dlambda_radial for a
plastic particle from (trial-stress/yield ratio, equivalent plastic strain,
log strain rate, homologous temperature).  Newton still converges to the same
relative residual, so the network changes only the iteration count; a
prediction outside (0, 1] is ignored and Newton starts from the radial value.

Everything runs in libweldform_gb300.so: synthetic states and their converged
increments, the FP32 training kernels (forward, backward, Adam), BF16
tensor-core inference.  This module only moves arrays.
"""
import ctypes as C

import numpy as np

from . import _abi
from .domain import lib

H = 64
NPARAM = H * 4 + H + H * H + H + H + 1     # 4545, WF_MLP_NPARAMS
_bound = False


def _L():
    global _bound
    L = lib()
    if not _bound:
        pf, pi = C.POINTER(C.c_float), C.POINTER(C.c_int32)
        L.wf_mlp_infer.restype = C.c_int
        L.wf_mlp_infer.argtypes = [pf, pf, C.c_int64, C.c_int, pf]
        L.wf_mlp_grad.restype = C.c_int
        L.wf_mlp_grad.argtypes = [pf, pf, pf, C.c_int64, pf, pf]
        L.wf_mlp_train.restype = C.c_int
        L.wf_mlp_train.argtypes = [pf, pf, pf, C.c_int64, C.c_int64, C.c_int64, C.c_float, pf]
        L.wf_mlp_synth.restype = C.c_int
        L.wf_mlp_synth.argtypes = [C.POINTER(_abi.WfMaterial), C.c_double, C.c_int64, C.c_uint64,
                                   C.c_double, pf, pf, pf, pi]
        L.wf_mlp_newton_iters.restype = C.c_int
        L.wf_mlp_newton_iters.argtypes = [C.POINTER(_abi.WfMaterial), C.c_double, pf, pf,
                                          C.c_int64, C.c_double, pi, pi, pf]
        L.wf_set_mlp_weights.restype = C.c_int
        L.wf_set_mlp_weights.argtypes = [C.c_void_p, pf]
        L.wf_get_return_map_log.restype = C.c_int
        L.wf_get_return_map_log.argtypes = [C.c_void_p, pf, pf, C.c_int64, C.POINTER(C.c_int64)]
        _bound = True
    return L


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _p(a, ct=C.c_float):
    return a.ctypes.data_as(C.POINTER(ct))


def _ck(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed (%d)" % (what, rc))


def init_params(seed=0):
    """He-style initialisation, packed W1, b1, W2, b2, W3, b3."""
    rng = np.random.default_rng(seed)
    W1 = rng.normal(0, np.sqrt(2.0 / 4), (H, 4))
    W2 = rng.normal(0, np.sqrt(2.0 / H), (H, H))
    W3 = rng.normal(0, np.sqrt(1.0 / H), H)
    return _f(np.concatenate([W1.ravel(), np.zeros(H), W2.ravel(), np.zeros(H), W3, [0.5]]))


def infer(params, X, tensor_cores=True):
    X = _f(X).reshape(-1, 4)
    Y = np.empty(len(X), np.float32)
    _ck(_L().wf_mlp_infer(_p(_f(params)), _p(X), len(X), 1 if tensor_cores else 0, _p(Y)),
        "wf_mlp_infer")
    return Y


def grad(params, X, Y):
    """(loss, gradient) of the mean squared error, from the training kernel."""
    X = _f(X).reshape(-1, 4)
    Y = _f(Y)
    g = np.empty(NPARAM, np.float32)
    loss = C.c_float()
    _ck(_L().wf_mlp_grad(_p(_f(params)), _p(X), _p(Y), len(X), _p(g), C.byref(loss)),
        "wf_mlp_grad")
    return float(loss.value), g


def train(params, X, Y, steps=3000, batch=2048, lr=3e-3):
    P = _f(params).copy()
    X = _f(X).reshape(-1, 4)
    Y = _f(Y)
    loss = C.c_float()
    _ck(_L().wf_mlp_train(_p(P), _p(X), _p(Y), len(X), int(steps), int(batch), float(lr),
                          C.byref(loss)), "wf_mlp_train")
    return P, float(loss.value)


def synth(mat, G, n, seed=2, rtol=1e-12):
    """Synthetic states and converged targets: (X, Y, states, radial iterations)."""
    X = np.empty((n, 4), np.float32)
    Y = np.empty(n, np.float32)
    S = np.empty((n, 4), np.float32)
    it = np.empty(n, np.int32)
    _ck(_L().wf_mlp_synth(C.byref(mat), float(G), int(n), int(seed), float(rtol), _p(X), _p(Y),
                          _p(S), _p(it, C.c_int32)), "wf_mlp_synth")
    return X, Y, S, it


def newton_iters(mat, G, params, states, rtol=1e-10):
    """Newton iterations per state from the network's start (params) or the
    radial start (params None): (iterations, used-network flags, increments)."""
    S = _f(states).reshape(-1, 4)
    n = len(S)
    it = np.empty(n, np.int32)
    used = np.empty(n, np.int32)
    dl = np.empty(n, np.float32)
    pp = None if params is None else _p(_f(params))
    _ck(_L().wf_mlp_newton_iters(C.byref(mat), float(G), pp, _p(S), n, float(rtol),
                                 _p(it, C.c_int32), _p(used, C.c_int32), _p(dl)),
        "wf_mlp_newton_iters")
    return it, used, dl


def train_jc_warm_start(mat, G, n_synth=262144, logged=None, steps=4000, batch=4096, lr=3e-3,
                        seed=2):
    """Trains the warm-start network on synthetic states (and, if given,
    pairs logged by the plain solver).  Returns (params, final loss)."""
    X, Y, _, _ = synth(mat, G, n_synth, seed=seed)
    if logged is not None and len(logged[0]):
        X = np.concatenate([X, logged[0]])
        Y = np.concatenate([Y, logged[1]])
    rng = np.random.default_rng(seed)
    order = rng.permutation(len(X))
    return train(init_params(seed), X[order], Y[order], steps=steps, batch=batch, lr=lr)


def set_domain_weights(dom, params):
    _ck(_L().wf_set_mlp_weights(dom.h, _p(_f(params))), "wf_set_mlp_weights")


def get_return_map_log(dom, cap):
    X = np.empty((cap, 4), np.float32)
    Y = np.empty(cap, np.float32)
    cnt = C.c_int64()
    _ck(_L().wf_get_return_map_log(dom.h, _p(X), _p(Y), int(cap), C.byref(cnt)),
        "wf_get_return_map_log")
    return X[:cnt.value], Y[:cnt.value]
