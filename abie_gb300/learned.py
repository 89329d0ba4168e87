"""Online training of the learned Radau15 predictor.

The batched Radau15 ensemble, run with the plain predictor, records for
every step reached in one attempt a training sample: the features of the
previous accepted step (its converged b coefficients scaled per order by
their largest magnitude s_k, the requested and actual step ratios, the
body's mass ratio, the log ratios of the scales) and the target (this
step's converged b minus the plain guess refine_bs made for it, per order
in units of s_k).  Each order's targets are normalised by a robust scale
tau_k (their 95th percentile magnitude; targets clipped at 20 tau_k), the
network is trained on the GPU with the library's own forward/backward
kernels (Adam), and is then switched on: later steps start from
E_k + s_k tau_k out_k instead of E_k, with the g coefficients made
consistent with that guess.  The convergence test of the corrector is
unchanged, so the solution is the same; only the number of corrector
iterations changes.
"""
import numpy as np

from .clibabie import CLibABIE

TARGETS = slice(32, 32 + 21)


def collect_samples(lib: CLibABIE, P, V, M, offs, G, years, capacity=1 << 20, seed=0):
    lib.mlp_init(seed, tau=None)
    lib.mlp_enable(False)
    lib.mlp_clear_samples()
    lib.mlp_set_capacity(capacity)
    res = lib.gr_ensemble(P, V, M, offs, G, 0.0, years, collect=True)
    return lib.mlp_samples(), res


def train_predictor(lib: CLibABIE, samples, steps=2000, batch=2048, lr=1e-3, seed=0,
                    holdout=0.1):
    S = np.array(samples, dtype=np.float32, copy=True)
    S = S[np.isfinite(S).all(axis=1)]
    # warps append samples in a run-dependent order: sort rows by content so
    # that training depends only on the sample set and the seed
    S = S[np.argsort(np.ascontiguousarray(S).view(np.dtype((np.void, S.shape[1] * 4))).ravel(),
                     kind="stable")]
    T = S[:, TARGETS].reshape(-1, 3, 7)          # [sample][d][k]
    tau = np.array([float(np.quantile(np.abs(T[:, :, k]), 0.95)) or 1.0 for k in range(7)])
    S[:, TARGETS] = np.clip(T / tau, -20.0, 20.0).reshape(-1, 21)
    rng = np.random.default_rng(seed)
    rng.shuffle(S)
    n_hold = int(len(S) * holdout)
    hold, train = S[:n_hold], S[n_hold:]
    lib.mlp_init(seed, tau=tau)
    lib.mlp_load_samples(train)
    last = lib.mlp_train(steps, batch, lr, seed)
    # held-out loss of the trained network vs the plain predictor (output 0)
    import ctypes
    L = lib.lib
    lib.mlp_load_samples(hold)
    L.abie_mlp_loss_grad.argtypes = [ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    loss = ctypes.c_double(0)
    grad = np.zeros(L.abie_mlp_n_params(), np.float32)
    L.abie_mlp_loss_grad(len(hold), grad.ctypes.data, ctypes.byref(loss))
    plain = float((hold[:, TARGETS] ** 2).mean())
    lib.mlp_enable(True)
    return {"samples": int(len(S)), "tau": tau.tolist(), "train_loss": last,
            "holdout_loss": loss.value, "holdout_loss_plain": plain}
