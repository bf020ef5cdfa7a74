"""CPU reference of the neural operator's layers — TEST INFRASTRUCTURE (the checker of
portlbm_gb300/csrc/plbm_nn.cu).  float64 numpy on the same bfloat16-rounded operands:

    conv3x3 (zero padding, NHWC, W[co][(ky*3+kx)*Cin+ci]) forward, data gradient, weight gradient,
    2x2 average pooling, nearest upsampling, and their adjoints.
"""
import numpy as np


def bf16_round(a):
    """Round float32/64 values to bfloat16 (nearest even) and return them as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _patches(x):
    """x [N,H,W,C] -> [N,H,W,9,C] neighbourhoods (ky, kx) with zero padding."""
    n, h, w, c = x.shape
    p = np.zeros((n, h + 2, w + 2, c))
    p[:, 1:-1, 1:-1] = x
    out = np.empty((n, h, w, 9, c))
    for ky in range(3):
        for kx in range(3):
            out[:, :, :, ky * 3 + kx] = p[:, ky:ky + h, kx:kx + w]
    return out


def conv_fwd(x, w, bias=None, relu=False):
    n, h, wd, cin = x.shape
    cout = w.shape[0]
    y = _patches(x).reshape(n * h * wd, 9 * cin) @ w.reshape(cout, 9 * cin).T
    if bias is not None:
        y = y + bias
    if relu:
        y = np.maximum(y, 0)
    return y.reshape(n, h, wd, cout)


def conv_dgrad(g, w, cin):
    """Gradient of the input: correlation of g with the flipped kernel, channels swapped."""
    n, h, wd, cout = g.shape
    wk = w.reshape(cout, 3, 3, cin)[:, ::-1, ::-1, :]                  # flip taps
    wt = np.transpose(wk, (3, 1, 2, 0)).reshape(cin, 9 * cout)         # [ci][(ky,kx,co)]
    return (_patches(g).reshape(n * h * wd, 9 * cout) @ wt.T).reshape(n, h, wd, cin)


def conv_wgrad(x, g):
    n, h, wd, cin = x.shape
    cout = g.shape[-1]
    gw = g.reshape(-1, cout).T @ _patches(x).reshape(n * h * wd, 9 * cin)
    return gw, g.reshape(-1, cout).sum(axis=0)


def pool2(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def up2(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)
