"""ORACLE / TEST INFRASTRUCTURE ONLY -- the checker of the learned-ordering
network's GPU kernels (circlecover_gb300/csrc/cc_mlp.cu), never used by the
product.

A float64 numpy restatement of the 10 -> 64 -> 64 -> 7 perceptron: forward
pass, mean summed binary cross-entropy, and its gradient by backpropagation
(itself checked against central finite differences by the CPU tests); plus a
BF16 emulation of the tensor-core inference (weights, inputs and hidden
activations rounded to bfloat16, sums in float32).  Parameter layout as in
include/circlecover_gb300.h: W1[10][64], b1[64], W2[64][64], b2[64],
W3[64][7], b3[7].
"""
import numpy as np

F, H, O = 10, 64, 7
SIZES = [("W1", F * H), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * O), ("b3", O)]
P = sum(n for _, n in SIZES)


def unpack(w):
    out, off = {}, 0
    for name, n in SIZES:
        out[name] = np.asarray(w[off:off + n], dtype=np.float64)
        off += n
    out["W1"] = out["W1"].reshape(F, H)
    out["W2"] = out["W2"].reshape(H, H)
    out["W3"] = out["W3"].reshape(H, O)
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def targets(labels):
    labels = np.asarray(labels, dtype=np.uint32)
    return ((labels[:, None] >> np.arange(O, dtype=np.uint32)) & 1).astype(np.float64)


def forward(w, x):
    p = unpack(w)
    x = np.asarray(x, dtype=np.float64)
    a1 = x @ p["W1"] + p["b1"]
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ p["W2"] + p["b2"]
    h2 = np.maximum(a2, 0.0)
    z = h2 @ p["W3"] + p["b3"]
    return z, (x, a1, h1, a2, h2)


def loss(w, x, labels):
    z, _ = forward(w, x)
    y = targets(labels)
    per = np.maximum(z, 0.0) - z * y + np.log1p(np.exp(-np.abs(z)))
    return per.sum() / len(z)


def gradient(w, x, labels):
    p = unpack(w)
    z, (x, a1, h1, a2, h2) = forward(w, x)
    y = targets(labels)
    n = len(z)
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / n
    g = {"W3": h2.T @ dz, "b3": dz.sum(0)}
    dh2 = (dz @ p["W3"].T) * (a2 > 0)
    g["W2"], g["b2"] = h1.T @ dh2, dh2.sum(0)
    dh1 = (dh2 @ p["W2"].T) * (a1 > 0)
    g["W1"], g["b1"] = x.T @ dh1, dh1.sum(0)
    return pack(g)


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def infer_bf16(w, x):
    """The tensor-core inference: bf16 inputs, weights and hidden activations,
    float32 sums, float32 biases."""
    p = {k: np.asarray(v, dtype=np.float32) for k, v in unpack(w).items()}
    h = bf16(x)
    h = np.maximum(h @ bf16(p["W1"]) + p["b1"], 0.0)
    h = np.maximum(bf16(h) @ bf16(p["W2"]) + p["b2"], 0.0)
    return bf16(h) @ bf16(p["W3"]) + p["b3"]
