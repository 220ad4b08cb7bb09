"""CPU float64 model of the SNR-screen MLP (test infrastructure, the checker of the GPU kernels).

Same feature map, standardisation, layer layout and BF16 rounding as the CUDA implementation
(gwfast_gb300/csrc/gwf_mlp.cu): the weights are used in BF16, and the hidden-to-hidden layers (both
widths multiples of 16, at most 256), which run on the tensor cores, also round their activation and
gradient operands to BF16 where they enter the products. The arithmetic is float64, so comparing
gradients shows the error of the GPU's FP32 accumulation (and the rare BF16 rounding it tips over).
"""
import numpy as np


def features(p):
    """p: (11, N) Fisher-order parameters -> (N, 11) raw features."""
    ra = p[4] - 2. * np.pi * p[7]
    return np.stack([np.log(p[0]), p[1], np.log(p[2]), np.cos(p[3]), np.sin(ra), np.cos(ra), np.cos(p[5]),
                     np.sin(2. * p[6]), np.cos(2. * p[6]), p[9], p[10]], axis=1)


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, hidden, layers):
    dims = [11] + [hidden] * layers + [1]
    Ws, bs, off = [], [], 0
    for k, m in zip(dims[:-1], dims[1:]):
        Ws.append(np.asarray(w[off:off + k * m]).reshape(k, m))
        off += k * m
    for m in dims[1:]:
        bs.append(np.asarray(w[off:off + m]))
        off += m
    return Ws, bs


def tensor_core_layer(l, n_layers, hidden):
    """The hidden-to-hidden layers run on the tensor cores (BF16 operands)."""
    return 1 <= l <= n_layers - 2 and hidden % 16 == 0 and hidden <= 256


def forward_backward(w, norm, p, target, hidden, layers):
    """Loss (mean squared error of ln SNR) and its gradient in the flat weight layout."""
    Ws, bs = unpack(np.asarray(w, dtype=np.float64), hidden, layers)
    Wq = [bf16(W.astype(np.float32)) for W in Ws]
    L = len(Wq)
    tc = [tensor_core_layer(l, L, hidden) for l in range(L)]
    x = (features(p).astype(np.float32).astype(np.float64) - norm[:11]) * norm[11:]
    acts, pres = [x], []
    a = x
    for l, (W, b) in enumerate(zip(Wq, bs)):
        z = (bf16(a) if tc[l] else a) @ W + b
        pres.append(z)
        a = z if l == len(Wq) - 1 else z / (1. + np.exp(-z))
        acts.append(a)
    y = a[:, 0]
    B = len(y)
    loss = np.mean((y - target) ** 2)
    dA = (2. * (y - target) / B)[:, None]
    gW, gb = [None] * len(Wq), [None] * len(Wq)
    for l in range(len(Wq) - 1, -1, -1):
        z = pres[l]
        if l == len(Wq) - 1:
            dZ = dA
        else:
            s = 1. / (1. + np.exp(-z))
            dZ = dA * s * (1. + z * (1. - s))
        gb[l] = dZ.sum(axis=0)
        if tc[l]:
            gW[l] = bf16(acts[l]).T @ bf16(dZ)
            dA = bf16(dZ) @ Wq[l].T
        else:
            gW[l] = acts[l].T @ dZ
            dA = dZ @ Wq[l].T
    return loss, np.concatenate([g.ravel() for g in gW] + [g.ravel() for g in gb])


def predict(w, norm, p, hidden, layers):
    """Predicted ln SNR (forward pass only) with the same roundings as the GPU's inference."""
    Ws, bs = unpack(np.asarray(w, dtype=np.float64), hidden, layers)
    Wq = [bf16(W.astype(np.float32)) for W in Ws]
    L = len(Wq)
    a = (features(p).astype(np.float32).astype(np.float64) - norm[:11]) * norm[11:]
    for l, (W, b) in enumerate(zip(Wq, bs)):
        z = (bf16(a) if tensor_core_layer(l, L, hidden) else a) @ W + b
        a = z if l == L - 1 else z / (1. + np.exp(-z))
    return a[:, 0]
