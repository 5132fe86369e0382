"""ORACLE — test infrastructure only.

The FP64 oracle of oracle/rl_oracle.py (rl_iterations and the radially
averaged branch of otf_on_grid with dtype=np.float64) written with torch
tensors, so that it runs on the GPU (cuFFT in double precision) for grids
whose float64 RL loop takes minutes on the host: 128x512x1024 with 20
iterations, 256x1024x1620 with 20 iterations.  Line for line the same
operations as the numpy restatement, which follows RichardsonLucy_GPU
(scopetools/cudadecon src/RL-Biggs-Andrews.cpp:282-367) and
dev_otfinterpolate's RA branch (src/RLgpuImpl.cu:238-273).

Pinned against the numpy FP64 oracle: tests/test_oracle_cpu.py runs both on
the same inputs (torch on the CPU) and requires agreement to 1e-12.
Only tests/ import this module; the product never does.
"""

from __future__ import annotations

import numpy as np

from .rl_oracle import FLT_EPS, kscales


def otf_on_grid(state, gx, gy, gz, device="cuda"):
    """rl_oracle.otf_on_grid(..., dtype=np.float64) for a radial OTF table,
    as a complex128 tensor of shape (gz, gy, gx//2+1)."""
    import torch
    if state.ny_otf != 1:
        raise ValueError("radially averaged OTF tables only")
    f64 = torch.float64
    kxs, kys, kzs = (float(v) for v in kscales(state, gx, gy, gz))
    nxh = gx // 2 + 1
    kx = torch.arange(nxh, dtype=f64, device=device) * kxs
    yy = torch.arange(gy, device=device)
    ky = torch.where(yy > gy >> 1, yy - gy, yy).to(f64) * kys
    zz = torch.arange(gz, device=device)
    kz = torch.where(zz > gz >> 1, zz - gz, zz).to(f64) * kzs
    otf = torch.from_numpy(np.ascontiguousarray(state.otf, np.complex128)).to(device)
    nzotf = float(state.nz_otf)
    kzi = torch.where(kz < 0, kz + nzotf, kz)
    nr = state.nx_otf
    kr = torch.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)  # (gy, nxh)
    out = torch.empty((gz, gy, nxh), dtype=torch.complex128, device=device)
    validr = kr < float(nr - 1)
    ir = torch.where(validr, torch.floor(kr), torch.zeros_like(kr)).to(torch.int64)
    ar = kr - ir.to(f64)
    ir1 = torch.clamp(ir + 1, max=nr - 1)
    # one kz plane at a time keeps the temporaries at (gy, nxh)
    for z in range(gz):
        KZ = kzi[z]
        if not (float(KZ) < nzotf and float(KZ) >= 0.0):
            out[z].zero_()
            continue
        iz = int(np.floor(float(KZ)))
        az = float(KZ) - iz
        iz1 = 0 if iz == state.nz_otf - 1 else iz + 1
        a = otf[:, iz] * (1.0 - az) + otf[:, iz1] * az  # (nr,)
        v = (1.0 - ar) * a[ir] + ar * a[ir1]
        out[z] = torch.where(validr, v, torch.zeros_like(v))
    return out


def rl_iterations(X0, raw, H, n_iters, lambdas=None, device="cuda"):
    """rl_oracle.rl_iterations(..., dtype=np.float64) on torch tensors.

    X0, raw: (nz, ny, nx) arrays or tensors; H: complex128 tensor on the
    half-spectrum grid.  Returns the final estimate (float64 tensor on
    `device`).  When lambdas is a list, the factor of each k > 1 is appended."""
    import torch
    f64 = torch.float64

    def dev(a):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(device=device, dtype=f64)

    X = dev(X0).clone()
    rawb = dev(raw)
    shape = tuple(X.shape)
    Hc = H.to(device=device, dtype=torch.complex128)
    Hcj = torch.conj(Hc)
    eps = FLT_EPS
    Xm1 = torch.zeros_like(X)
    G1 = torch.zeros_like(X)
    G2 = torch.zeros_like(X)

    def conv(a, conj):
        F = torch.fft.rfftn(a)
        F *= Hcj if conj else Hc
        return torch.fft.irfftn(F, s=shape)

    for k in range(n_iters):
        if k > 1:
            num = float(torch.sum(G1 * G2))
            den = float(torch.sum(G2 * G2))
            lam = num / (den + FLT_EPS)
            lam = 1.0 if 1.0 < lam else lam
            lam = 0.0 if lam < 0.0 else lam
            if lambdas is not None:
                lambdas.append(lam)
            Y = X + lam * (X - Xm1)
            Y = torch.where(Y > 0, Y, torch.zeros_like(Y))
        else:
            Y = X.clone()
        Xm1 = X
        if k > 0:
            G2 = G1
        CC = conv(Y, False)
        CC = torch.where(torch.abs(CC) > 0, CC, torch.full_like(CC, eps))
        CC = rawb / CC + eps
        CC = torch.clamp(CC, -10.0, 10.0)
        CC = conv(CC, True)
        X = CC * Y
        X = torch.where(X > 0, X, torch.zeros_like(X))
        G1 = X - Y
        del CC
    return X
