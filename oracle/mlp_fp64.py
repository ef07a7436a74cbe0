"""FP64 NumPy restatement of the transmit-field surrogate network (test infrastructure only):
random Fourier features -> 4 x (Linear 256 + SiLU) -> Linear n_out.  The training loss is
mean_batch |sum_j (o_2j + i o_2j+1) c_j - y|^2 over analytic carriers c_j (the quantities that
fsg_surrogate_inputs writes per sample as aux = [c_0 .. c_4, y], complex pairs).  Used to
check the outputs and gradients of the GPU training and inference kernels."""

import numpy as np


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def features(u, bmat):
    t = u @ bmat.T
    return np.concatenate([np.sin(2 * np.pi * t), np.cos(2 * np.pi * t)], axis=1)


def forward(u, bmat, W, b):
    a = features(u, bmat)
    acts, zs = [a], []
    for w, bb in zip(W[:-1], b[:-1]):
        z = a @ w.T + bb
        a = silu(z)
        zs.append(z)
        acts.append(a)
    out = a @ W[-1].T + b[-1]
    return out, acts, zs


AUX = 12  # floats per training row: carriers c_0 .. c_4, target y (complex pairs)


def carriers(samples, n_elements, pitch, c, n_carriers=5):
    """The analytic carriers of the surrogate at samples (n, 4) = (x, z, f, theta): the plane
    wave exp(i k (x sin th + z cos th - xmin)); the waves of the aperture ends
    exp(i k (r_edge + x_edge sin th - xmin)), x_edge half a pitch outside the end elements; the
    grating lobes m = -1, +1, exp(i k (x sin th_m + z cos th_m - xmin)) with
    sin th_m = sin th + m lambda / pitch, zero where |sin th_m| >= 1.
    xmin = min(x_0 sin th, x_{E-1} sin th), k = 2 pi f / c."""
    x, z, f, th = (samples[:, i] for i in range(4))
    st, ct = np.sin(th), np.cos(th)
    x0 = -0.5 * (n_elements - 1) * pitch
    xmin = np.minimum(x0 * st, -x0 * st)
    k = 2.0 * np.pi * f / c
    paths, on = [x * st + z * ct - xmin], [np.ones_like(x, dtype=bool)]
    for xe in (x0 - 0.5 * pitch, -x0 + 0.5 * pitch):
        paths.append(np.sqrt((x - xe) ** 2 + z ** 2) + xe * st - xmin)
        on.append(np.ones_like(x, dtype=bool))
    lp = c / f / pitch
    for m in (-1, 1):
        sm = st + m * lp
        paths.append(x * sm + z * np.sqrt(np.maximum(0.0, 1.0 - sm * sm)) - xmin)
        on.append(np.abs(sm) < 1.0)
    return np.stack([np.where(on[j], np.exp(1j * k * paths[j]), 0.0) for j in range(n_carriers)], axis=-1)


def backprop(d, acts, zs, W):
    """Gradients of every weight and bias given the head's output gradient d (n x n_out)."""
    gW = [None] * len(W)
    gb = [None] * len(W)
    gW[-1] = d.T @ acts[-1]
    gb[-1] = d.sum(0)
    da = d @ W[-1]
    for layer in range(len(W) - 2, -1, -1):
        dz = da * silu_grad(zs[layer])
        gW[layer] = dz.T @ acts[layer]
        gb[layer] = dz.sum(0)
        da = dz @ W[layer]
    return gW, gb


def carrier_field(out, aux):
    """p = sum_j (o_2j + i o_2j+1) c_j for the carriers stored in aux."""
    nc = out.shape[1] // 2
    c = aux[:, 0:2 * nc:2] + 1j * aux[:, 1:2 * nc:2]
    return ((out[:, 0::2] + 1j * out[:, 1::2]) * c).sum(1)


def target(aux):
    return aux[:, AUX - 2] + 1j * aux[:, AUX - 1]


def carrier_loss_and_grads(u, aux, bmat, W, b):
    """Loss mean |p - y|^2 and its gradients, y = target(aux)."""
    out, acts, zs = forward(u, bmat, W, b)
    n = u.shape[0]
    nc = out.shape[1] // 2
    err = carrier_field(out, aux) - target(aux)
    loss = float(np.mean(np.abs(err) ** 2))
    c = aux[:, 0:2 * nc:2] + 1j * aux[:, 1:2 * nc:2]
    w = np.conj(err)[:, None] * c
    d = np.zeros_like(out)
    d[:, 0::2] = 2.0 / n * w.real
    d[:, 1::2] = -2.0 / n * w.imag
    gW, gb = backprop(d, acts, zs, W)
    return loss, gW, gb
