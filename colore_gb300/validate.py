"""Field checks of the FP32 path against the plain FP64 path on the same GPU.

Both paths draw every Fourier mode from the same Philox stream, so their
Gaussian fields and potentials differ only by arithmetic.  field_errors()
compares them where they live, on the device, with torch as the FP64
calculator:

  rel_rms   sqrt(sum (a - b)^2 / sum b^2) over the N^3 cells;
  pk        the power spectrum of each field in spherical shells of |k|, one
            fundamental mode wide (shell i holds i - 1/2 <= |k|/k_f < i + 1/2,
            i = 1 .. N/2), from torch's FP64 rfftn with the Hermitian weight 2
            on the planes 0 < kx < N/2; pk_rel_err is |P32 / P64 - 1| per
            shell and pk_max_rel_err its maximum.

Used by the tests and by the benchmark line (the metric is gated on the
per-shell P(k) error).  Needs torch and a CUDA device.
"""
import numpy as np


def _torch():
    import torch
    return torch


def pk_shells(x, chunk=64):
    """Shell-summed |FFT(x)|^2 and mode counts of an (N, N, N) float64 CUDA
    tensor, shells i = round(|k| / k_f) for i = 0 .. N/2 (float64 tensors)."""
    torch = _torch()
    n = x.shape[0]
    f = torch.fft.rfftn(x)
    nb = n // 2 + 1
    kz_all = torch.fft.fftfreq(n, d=1.0 / n, device=x.device, dtype=torch.float64)
    ky = kz_all.view(1, n, 1)
    kx = torch.arange(n // 2 + 1, device=x.device, dtype=torch.float64).view(1, 1, -1)
    w = torch.full((n // 2 + 1,), 2.0, device=x.device, dtype=torch.float64)
    w[0] = 1.0
    if n % 2 == 0:
        w[-1] = 1.0
    w = w.view(1, 1, -1)
    psum = torch.zeros(nb, device=x.device, dtype=torch.float64)
    cnt = torch.zeros(nb, device=x.device, dtype=torch.float64)
    for z0 in range(0, n, chunk):
        z1 = min(n, z0 + chunk)
        kz = kz_all[z0:z1].view(-1, 1, 1)
        kk = torch.sqrt(kz * kz + ky * ky + kx * kx)
        b = torch.floor(kk + 0.5).to(torch.int64)
        fz = f[z0:z1]
        p = (fz.real ** 2 + fz.imag ** 2) * w
        ww = torch.broadcast_to(w, p.shape)
        keep = b < nb
        psum += torch.bincount(b[keep], weights=p[keep], minlength=nb)[:nb]
        cnt += torch.bincount(b[keep], weights=ww[keep], minlength=nb)[:nb]
        del kk, b, p, ww, keep
    del f
    return psum, cnt


def compare(a32_padded, b64):
    """Errors of one FP32 padded grid (N, N, 2(N/2+1)) against the FP64
    unpadded (N, N, N) grid, both CUDA tensors: dict with rel_rms,
    pk_rel_err (per shell 1 .. N/2) and pk_max_rel_err."""
    torch = _torch()
    n = b64.shape[0]
    num = 0.0
    den = 0.0
    for z0 in range(0, n, 64):
        a = a32_padded[z0:z0 + 64, :, :n].to(torch.float64)
        b = b64[z0:z0 + 64]
        num += float(((a - b) ** 2).sum())
        den += float((b * b).sum())
        del a
    a = a32_padded[:, :, :n].to(torch.float64)
    pa, _ = pk_shells(a)
    del a
    pb, cnt = pk_shells(b64)
    rel = (pa[1:] / pb[1:] - 1.0).abs().cpu().numpy()
    return {"rel_rms": float(np.sqrt(num / den)), "pk_rel_err": rel, "pk_max_rel_err": float(rel.max()),
            "pk_modes": cnt[1:].cpu().numpy()}


def field_errors(m32, m64, which=(0, 1)):
    """FP32 context m32 (after create_cartesian_fields) against FP64 context
    m64 (after create_cartesian_fields) on the same configuration: a dict
    per grid (0: Gaussian density, 1: potential) as compare() returns."""
    torch = _torch()
    from . import grid_shape
    n = m32.n
    out = {}
    for w in which:
        a = torch.empty(grid_shape(n), dtype=torch.float32, device="cuda")
        m32.grid(w, out=a)
        b = torch.empty((n, n, n), dtype=torch.float64, device="cuda")
        m64.density(w, out=b)
        torch.cuda.synchronize()
        out[w] = compare(a, b)
        del a, b
        torch.cuda.empty_cache()
    return out
