"""CPU oracle of the learned TENO stencil selector (test infrastructure only).

The selector has no counterpart in the reference: this module restates the
network the GPU kernels implement so that tests can check them.

* forward / backward of the 96-64-64-32 MLP (GELU, tanh form) with a
  softmax cross-entropy per 8-class head, in float64;
* the tensor-core inference path emulated in numpy: features and weights
  rounded to BF16 (nearest even), FP32 accumulation, bias + GELU in FP32,
  the activation rounded to BF16 before the next layer;
* the feature construction from a state and the TENO stencils.

Only tests and the benchmark's checks import this module.
"""

import numpy as np

NV, PER_VAR, HID, NCLS = 4, 24, 64, 8
IN, OUT = NV * PER_VAR, NV * NCLS
MR = 19
FLAT_RANGE = np.float32(1e-5)  # ranges up to this count as zero (selector.cuh)
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * OUT
N_PARAMS = OFF_B3 + OUT

_C = np.sqrt(2.0 / np.pi)


def unpack(p):
    p = np.asarray(p)
    return (p[OFF_W1:OFF_B1].reshape(IN, HID), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(HID, HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(HID, OUT), p[OFF_B3:N_PARAMS])


def pack(W1, b1, W2, b2, W3, b3):
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(_C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(_C * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _C * (1.0 + 3.0 * 0.044715 * x * x)


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, dtype=np.float64))
    X = np.asarray(X, dtype=np.float64)
    Z1 = X @ W1 + b1
    A1 = gelu(Z1)
    Z2 = A1 @ W2 + b2
    A2 = gelu(Z2)
    Z3 = A2 @ W3 + b3
    return Z1, A1, Z2, A2, Z3


def loss_and_grad(p, X, Y):
    """Mean cross-entropy over rows and heads, and its gradient (packed)."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, dtype=np.float64))
    X = np.asarray(X, dtype=np.float64)
    Z1, A1, Z2, A2, Z3 = forward(p, X)
    n = X.shape[0]
    z = Z3.reshape(n, NV, NCLS)
    z = z - z.max(axis=2, keepdims=True)
    e = np.exp(z)
    s = e.sum(axis=2, keepdims=True)
    prob = e / s
    Y = np.asarray(Y, dtype=np.int64).reshape(n, NV)
    onehot = np.zeros_like(prob)
    np.put_along_axis(onehot, Y[:, :, None], 1.0, axis=2)
    loss = float(np.mean(np.log(s[:, :, 0]) - np.take_along_axis(z, Y[:, :, None], axis=2)[:, :, 0]))
    dZ3 = ((prob - onehot) / (n * NV)).reshape(n, OUT)
    dW3 = A2.T @ dZ3
    db3 = dZ3.sum(axis=0)
    dZ2 = (dZ3 @ W3.T) * gelu_grad(Z2)
    dW2 = A1.T @ dZ2
    db2 = dZ2.sum(axis=0)
    dZ1 = (dZ2 @ W2.T) * gelu_grad(Z1)
    dW1 = X.T @ dZ1
    db1 = dZ1.sum(axis=0)
    return loss, pack(dW1, db1, dW2, db2, dW3, db3)


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return (b.astype(np.uint32) << 16).view(np.float32)


def infer_bf16(p, X):
    """Logits as the tensor-core path computes them (up to summation order)."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(p, dtype=np.float32))
    x = bf16(X).astype(np.float64)
    z1 = (x @ bf16(W1).astype(np.float64)).astype(np.float32) + b1
    a1 = bf16(gelu(z1.astype(np.float64)).astype(np.float32)).astype(np.float64)
    z2 = (a1 @ bf16(W2).astype(np.float64)).astype(np.float32) + b2
    a2 = bf16(gelu(z2.astype(np.float64)).astype(np.float32)).astype(np.float64)
    return (a2 @ bf16(W3).astype(np.float64)).astype(np.float32) + b3


def class_of_mask(mask):
    mask = np.asarray(mask).astype(np.int64)
    return np.where(mask & 1, 0, (mask >> 1) & 7)


def mask_of_class(c):
    c = np.asarray(c).astype(np.int64)
    return np.where(c == 0, 1, c << 1)


def predict(logits, threshold):
    """Per row and head: (predicted TENO mask | 0x80 when confident)."""
    z = np.asarray(logits, dtype=np.float64).reshape(-1, NV, NCLS)
    arg = z.argmax(axis=2)
    s = np.exp(z - z.max(axis=2, keepdims=True)).sum(axis=2)
    conf = s <= 1.0 / threshold
    return (mask_of_class(arg) | np.where(conf, 0x80, 0)).astype(np.uint8)


def features(U, off_stencils, stencils, cells=None):
    """Feature rows [len(cells)][96] from a state U [n][4] (FP64) and the
    TENO stencils in the reference layout (4 stencils per cell, target
    first, empty stencils where a face is on the boundary): per variable the
    19 central-stencil differences divided by their range, the scaled log10
    of the range, the directional ranges relative to it and a zero; ranges
    up to FLAT_RANGE count as zero."""
    U = np.asarray(U, dtype=np.float64)
    n = U.shape[0]
    cells = np.arange(n) if cells is None else np.asarray(cells)
    Uf = U.astype(np.float32)
    out = np.zeros((len(cells), IN), dtype=np.float32)
    one = np.float32(1.0)
    for r, c in enumerate(cells):
        so, se = off_stencils[4 * c], off_stencils[4 * c + 1]
        nb = stencils[so + 1:se]
        for v in range(NV):
            uc = Uf[c, v]
            row = out[r, v * PER_VAR:(v + 1) * PER_VAR]
            d = (Uf[nb, v] - uc).astype(np.float32)
            lo = min(np.float32(0.0), d.min())
            hi = max(np.float32(0.0), d.max())
            r0 = np.float32(hi - lo)
            r0 = r0 if r0 > FLAT_RANGE else np.float32(0.0)
            inv = one / r0 if r0 > 0 else np.float32(0.0)
            row[:MR] = d * inv
            row[MR] = np.clip((np.log10(np.float32(r0)) + 6.0) / 6.0, -1.0, 1.0) if r0 > 0 else -1.0
            for s in range(1, 4):
                a, b = off_stencils[4 * c + s], off_stencils[4 * c + s + 1]
                if b == a:
                    row[MR + s] = -1.0
                    continue
                ds = (Uf[stencils[a + 1:b], v] - uc).astype(np.float32)
                rs = np.float32(max(np.float32(0.0), ds.max()) - min(np.float32(0.0), ds.min()))
                if r0 > 0:
                    row[MR + s] = min(np.float32(rs * inv), np.float32(4.0)) * np.float32(0.25)
                else:
                    row[MR + s] = 1.0 if rs > FLAT_RANGE else 0.0
            row[PER_VAR - 1] = 0.0
    return out
