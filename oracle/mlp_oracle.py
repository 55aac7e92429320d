"""FP64 numpy restatement of the warm-start MLP (32 -> 128 x4 -> 3, ReLU, MSE).

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward / backward kernels.
The forward pass uses the BF16-rounded weights the GPU uses and FP32 biases; the
gradients returned are those of the mean-squared error w.r.t. every parameter, in
the library's layout (per layer W[out][in] then b[out]).
"""
import numpy as np

DIMS = [32, 128, 128, 128, 128, 3]


def bf16_round(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(params: np.ndarray):
    Ws, bs, at = [], [], 0
    for l in range(5):
        o, i = DIMS[l + 1], DIMS[l]
        Ws.append(params[at:at + o * i].reshape(o, i))
        at += o * i
        bs.append(params[at:at + o])
        at += o
    return Ws, bs


def _round(a, on):
    return bf16_round(np.asarray(a, np.float32)).astype(np.float64) if on else a


def forward(params, X, bf16_acts: bool = False):
    """Layer inputs and the output.  bf16_acts: the input and every hidden activation rounded to
    BF16, as the tensor-core engine feeds them to its GEMMs."""
    Ws, bs = unpack(params)
    acts = [_round(np.asarray(X, np.float64), bf16_acts)]
    for l in range(5):
        z = acts[-1] @ bf16_round(Ws[l]).astype(np.float64).T + bs[l].astype(np.float64)
        acts.append(_round(np.maximum(z, 0), bf16_acts) if l < 4 else z)
    return acts


def gradients(params, X, T, bf16_acts: bool = False):
    """MSE gradients; bf16_acts also rounds every layer's output gradient dZ to BF16 (the
    tensor-core engine's GEMM operand) before it is used."""
    Ws, bs = unpack(params)
    acts = forward(params, X, bf16_acts)
    P = X.shape[0]
    d = 2.0 * (acts[-1] - np.asarray(T, np.float64)) / (P * 3)
    loss = float(np.mean((acts[-1] - T) ** 2))
    gW, gb = [None] * 5, [None] * 5
    d = _round(d, bf16_acts)
    for l in range(4, -1, -1):
        if l < 4:
            d = _round(d * (acts[l + 1] > 0), bf16_acts)
        gW[l] = d.T @ acts[l]
        gb[l] = d.sum(0)
        d = d @ bf16_round(Ws[l]).astype(np.float64)
    out = []
    for l in range(5):
        out.append(gW[l].ravel())
        out.append(gb[l])
    return np.concatenate(out), loss
