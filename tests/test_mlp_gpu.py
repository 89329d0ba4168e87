"""The learned predictor's GPU kernels (BF16 mma.sync, FP32 accumulation)
against the CPU checker oracle/mlp_ref.py, which rounds the same operands
to bfloat16 and sums in float64: outputs to 1e-4 and every gradient tensor
to 1e-3 relative (L2 norms); training lowers the loss."""
import ctypes as C

import numpy as np
import pytest

import oracle.mlp_ref as R

pytestmark = pytest.mark.gpu


def _lib(clib):
    L = clib.lib
    L.abie_mlp_init.argtypes = [C.c_int, C.c_void_p]
    L.abie_mlp_set_params.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    L.abie_mlp_get_params.argtypes = [C.c_void_p, C.c_int]
    L.abie_mlp_load_samples.argtypes = [C.c_void_p, C.c_longlong]
    L.abie_mlp_forward.argtypes = [C.c_longlong, C.c_void_p]
    L.abie_mlp_loss_grad.argtypes = [C.c_longlong, C.c_void_p, C.c_void_p]
    L.abie_mlp_train.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p]
    return L


def _random_params(rng):
    p = [rng.normal(0, 0.2, (R.HID, R.IN)), rng.normal(0, 0.1, R.HID),
         rng.normal(0, 0.1, (R.HID, R.HID)), rng.normal(0, 0.1, R.HID),
         rng.normal(0, 0.1, (R.OUT_PAD, R.HID)), rng.normal(0, 0.1, R.OUT_PAD)]
    return p, np.concatenate([a.reshape(-1) for a in p]).astype(np.float32)


def _samples(rng, rows):
    X = np.zeros((rows, R.IN), np.float32)
    X[:, :30] = rng.normal(size=(rows, 30))
    T = np.zeros((rows, R.OUT_PAD), np.float32)
    T[:, :R.OUT] = rng.normal(size=(rows, R.OUT))
    return X, T, np.ascontiguousarray(np.concatenate([X, T], axis=1))


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300)


def test_forward_and_gradients_match_checker(clib):
    L = _lib(clib)
    rng = np.random.default_rng(1)
    params, flat = _random_params(rng)
    assert L.abie_mlp_set_params(flat.ctypes.data, flat.size, None) == 0
    rows = 200  # several CTAs of 64 and a ragged last one
    X, T, S = _samples(rng, rows)
    assert L.abie_mlp_load_samples(S.ctypes.data, rows) == 0
    Y = np.zeros((rows, R.OUT_PAD), np.float32)
    assert L.abie_mlp_forward(rows, Y.ctypes.data) == 0
    # the checker uses the same (float32) parameters
    p32 = R.unpack(flat)
    Yref, _ = R.forward(p32, X.astype(np.float64))
    assert _rel(Y, Yref) <= 1e-4
    g = np.zeros(R.N_PARAMS, np.float32)
    loss = C.c_double(0)
    assert L.abie_mlp_loss_grad(rows, g.ctypes.data, C.byref(loss)) == 0
    lref, gref = R.loss_and_grads(p32, X.astype(np.float64), T.astype(np.float64))
    assert abs(loss.value - lref) <= 1e-4 * lref
    gg = R.unpack(g)
    for name, a, b in zip(["W1", "b1", "W2", "b2", "W3", "b3"], gg, gref):
        assert _rel(a, b) <= 1e-3, name


def test_training_lowers_loss(clib):
    L = _lib(clib)
    rng = np.random.default_rng(2)
    assert L.abie_mlp_init(7, None) == 0
    rows = 4096
    X = np.zeros((rows, R.IN), np.float32)
    X[:, :30] = rng.normal(size=(rows, 30))
    A = rng.normal(0, 0.3, (30, R.OUT))
    T = np.zeros((rows, R.OUT_PAD), np.float32)
    T[:, :R.OUT] = np.tanh(X[:, :30] @ A)
    S = np.ascontiguousarray(np.concatenate([X, T], axis=1))
    assert L.abie_mlp_load_samples(S.ctypes.data, rows) == 0
    grad = np.zeros(R.N_PARAMS, np.float32)  # kept alive across the calls
    l0 = C.c_double(0)
    assert L.abie_mlp_loss_grad(rows, grad.ctypes.data, C.byref(l0)) == 0
    last = C.c_double(0)
    assert L.abie_mlp_train(400, 256, 3e-3, 5, C.byref(last)) == 0
    l1 = C.c_double(0)
    assert L.abie_mlp_loss_grad(rows, grad.ctypes.data, C.byref(l1)) == 0
    assert l1.value < 0.2 * l0.value, (l0.value, l1.value)
