"""CPU oracle of the learned-guess network -- test infrastructure only.

The reference has no learned component; this restates, in float64 numpy, what
the library's CUDA kernels (mantle_convection_lab_gb300/csrc/cuda/k_cnn.cu)
compute, so that their forward pass, gradients and Adam step can be checked:

- parameters are one flat array, layer by layer: W[cout][cin][3][3], b[cout];
- layer l: z = b + sum_c sum_k W[o][c][k] * x[c][y+ky-1][x+kx-1] (zero padding),
  then ReLU on every layer but the last;
- the forward pass uses the weights rounded to bfloat16 (round to nearest
  even), biases in full precision, and -- as the tensor-core convolutions
  stage them -- each layer's input rounded to float32 and then to bfloat16;
- loss = mean((y - t)^2), gradients by back-propagation with respect to the
  rounded weights (applied to the FP32 master weights by Adam); the gradient
  passed back through a convolution is rounded to bfloat16 the same way, the
  weight gradient uses the unrounded activations and gradients;
- Adam: beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected, in float32.

The oracle is pinned by finite differences (tests/test_cnn_oracle.py).
"""
import numpy as np


def bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def bf16_in(a, jitter=None):
    """A convolution input as the tensor-core kernels stage it: float32, then
    bfloat16.  With jitter (a numpy Generator) each value is first moved by up
    to 2^-19 relative (16 float32 ulps, the rounding of an FP32 sum of a few
    hundred products), as another FP32 summation order would move it; the
    spread of results over jitters measures how far BF16 rounding flips can
    carry an FP32 computation from this float64 one."""
    a = np.asarray(a, np.float64)
    if jitter is not None:
        a = a * (1.0 + jitter.uniform(-1.0, 1.0, a.shape) * 2.0 ** -19)
    return bf16(a.astype(np.float32)).astype(np.float64)


def layer_shapes(cin, width, depth, cout):
    return [(cout if l == depth - 1 else width, cin if l == 0 else width) for l in range(depth)]


def unpack(params, shapes):
    out, off = [], 0
    for co, ci in shapes:
        nw = co * ci * 9
        W = params[off:off + nw].reshape(co, ci, 3, 3)
        b = params[off + nw:off + nw + co]
        out.append((W, b))
        off += nw + co
    assert off == params.size
    return out


def conv(x, W, b):
    B, C, H, Wd = x.shape
    xp = np.pad(x, ((0, 0), (0, 0), (1, 1), (1, 1)))
    out = np.zeros((B, W.shape[0], H, Wd))
    for ky in range(3):
        for kx in range(3):
            out += np.einsum("oc,bcyx->boyx", W[:, :, ky, kx], xp[:, :, ky:ky + H, kx:kx + Wd], optimize=True)
    return out + b[None, :, None, None]


def forward(params, shapes, x, quantize=True, jitter=None):
    """Activations a[0] = x, a[l+1] = layer l output (float64)."""
    layers = unpack(np.asarray(params, np.float32), shapes)
    a = [np.asarray(x, np.float64)]
    for l, (W, b) in enumerate(layers):
        Wq = (bf16(W) if quantize else W).astype(np.float64)
        z = conv(bf16_in(a[-1], jitter if l > 0 else None) if quantize else a[-1], Wq, b.astype(np.float64))
        a.append(np.maximum(z, 0.0) if l + 1 < len(layers) else z)
    return a


def loss_and_grad(params, shapes, x, t, quantize=True, jitter=None):
    layers = unpack(np.asarray(params, np.float32), shapes)
    a = forward(params, shapes, x, quantize, jitter)
    y = a[-1]
    t = np.asarray(t, np.float64)
    n = y.size
    loss = float(np.sum((y - t) ** 2) / n)
    gz = 2.0 * (y - t) / n
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        Wq = (bf16(W) if quantize else W).astype(np.float64)
        ap = np.pad(a[l], ((0, 0), (0, 0), (1, 1), (1, 1)))
        H, Wd = a[l].shape[2:]
        dW = np.zeros(W.shape)
        for ky in range(3):
            for kx in range(3):
                dW[:, :, ky, kx] = np.einsum("boyx,bcyx->oc", gz, ap[:, :, ky:ky + H, kx:kx + Wd], optimize=True)
        grads[l] = np.concatenate([dW.ravel(), gz.sum(axis=(0, 2, 3))])
        if l > 0:
            gp = np.pad(bf16_in(gz, jitter) if quantize else gz, ((0, 0), (0, 0), (1, 1), (1, 1)))
            ga = np.zeros(a[l].shape)
            for ky in range(3):
                for kx in range(3):
                    ga += np.einsum("oc,boyx->bcyx", Wq[:, :, ky, kx],
                                    gp[:, :, 2 - ky:2 - ky + H, 2 - kx:2 - kx + Wd], optimize=True)
            gz = ga * (a[l] > 0)
    return loss, np.concatenate(grads)


def adam(w, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step in float32; returns (w, m, v)."""
    f = np.float32
    w, g, m, v = (np.asarray(z, np.float32) for z in (w, g, m, v))
    m = f(b1) * m + f(1 - b1) * g
    v = f(b2) * v + f(1 - b2) * g * g
    c1 = f(1) - f(b1) ** f(t)
    c2 = f(1) - f(b2) ** f(t)
    w = w - f(lr) * (m / c1) / (np.sqrt(v / c2) + f(eps))
    return w, m, v
