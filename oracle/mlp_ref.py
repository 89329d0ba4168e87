"""CPU checker for the learned Radau15 predictor -- TEST INFRASTRUCTURE ONLY.

A float64 NumPy statement of the network the library runs on the GPU:

    H1 = relu(bf16(X)  @ bf16(W1)^T + b1)      X: rows x 32 (30 features, zero padded)
    H2 = relu(bf16(H1) @ bf16(W2)^T + b2)      W1: 128 x 32, W2: 128 x 128
    Y  =      bf16(H2) @ bf16(W3)^T + b3       W3: 32 x 128 (21 outputs, zero padded)
    loss = sum over rows and the 21 outputs of (Y - T)^2 / (rows * 21)

Gradients follow the GPU's definition: the output delta and the hidden
deltas are rounded to bfloat16 before they enter the next product, and the
bias gradients are the column sums of those rounded deltas.

Every tensor-core operand is rounded to bfloat16 (round to nearest even)
exactly where the GPU rounds it, products are exact and sums are carried in
float64, so the GPU's FP32 accumulation is the only remaining difference.
"""
import numpy as np

IN, HID, OUT, OUT_PAD = 32, 128, 21, 32


def bf16(a):
    """Round float32/float64 values to bfloat16 (nearest even), returned as float64."""
    a32 = np.asarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(params, X):
    W1, b1, W2, b2, W3, b3 = params
    A0 = bf16(X)
    Z1 = A0 @ bf16(W1).T + b1
    H1 = np.maximum(Z1, 0.0)
    A1 = bf16(H1)
    Z2 = A1 @ bf16(W2).T + b2
    H2 = np.maximum(Z2, 0.0)
    A2 = bf16(H2)
    Y = A2 @ bf16(W3).T + b3
    return Y, (A0, Z1, A1, Z2, A2)


def loss_and_grads(params, X, T):
    """Mean squared error over the first OUT outputs and its gradients."""
    W1, b1, W2, b2, W3, b3 = params
    rows = X.shape[0]
    Y, (A0, Z1, A1, Z2, A2) = forward(params, X)
    D = np.zeros_like(Y)
    D[:, :OUT] = Y[:, :OUT] - T[:, :OUT]
    loss = float((D[:, :OUT] ** 2).sum() / (rows * OUT))
    dY = 2.0 * D / (rows * OUT)
    # the GPU feeds bf16(dY) and bf16 copies of activations to the tensor cores
    dYb = bf16(dY)
    dW3 = dYb.T @ A2
    db3 = dYb.sum(0)
    dA2 = dYb @ bf16(W3)
    dZ2 = dA2 * (Z2 > 0)
    dZ2b = bf16(dZ2)
    dW2 = dZ2b.T @ A1
    db2 = dZ2b.sum(0)
    dA1 = dZ2b @ bf16(W2)
    dZ1 = dA1 * (Z1 > 0)
    dZ1b = bf16(dZ1)
    dW1 = dZ1b.T @ A0
    db1 = dZ1b.sum(0)
    return loss, (dW1, db1, dW2, db2, dW3, db3)


def unpack(flat):
    """Split the library's flat FP32 parameter vector (W1 b1 W2 b2 W3 b3)."""
    flat = np.asarray(flat, dtype=np.float64)
    shapes = [(HID, IN), (HID,), (HID, HID), (HID,), (OUT_PAD, HID), (OUT_PAD,)]
    out, k = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(flat[k:k + n].reshape(s))
        k += n
    return out


N_PARAMS = HID * IN + HID + HID * HID + HID + OUT_PAD * HID + OUT_PAD
