"""Seeded synthetic survey inputs in the reference's file formats.

Writes the four files the reference program reads from its working directory:

* ``FDTD_setup.in`` -- 8 lines (ModelingSetup.cpp:51-59)
* ``Cond.bin``      -- float64 conductivity, N*M*L values, x fastest (ModelingSetup.cpp:201-209)
* ``Receiver.in``   -- time window, component flags, receiver positions (LoadRxTxPos.cpp:51-84)
* ``Transmitter.in``-- transmitter records ``id ort BipoLen x y z [azi dip] nr rx...`` (LoadRxTxPos.cpp:134-200)

The named cases reproduce the survey configurations with seeded synthetic
models (no measured data is involved).  Every case is a plain dictionary so a
test can derive variants from it.
"""
from __future__ import annotations

import copy
import math
import os

import numpy as np

MU0 = 4 * math.pi * 1e-7

# --------------------------------------------------------------------------- grid helpers


def grid_axes(c):
    """Cell sizes and node coordinates exactly as ModelingSetup.cpp:100-187 builds them."""
    ALx2, ALx1, Nx, ARx1, ARx2 = c["xsplit"]
    Ay2, Ay1, Ny = c["ysplit"]
    Az2, Az1, Nz = c["zsplit"]
    a1, a2 = c["arg1"], c["arg2"]
    dxm, dym, dzm = c["dmin"]
    L = ALx2 + ALx1 + ARx2 + ARx1 + Nx
    M = 2 * (Ay2 + Ay1) + Ny
    N = Nz + Az2 + Az1
    AL = ALx2 + ALx1
    dx = np.zeros(L)
    dx[AL:AL + Nx] = dxm
    for i in range(AL - 1, ALx2 - 1, -1):
        dx[i] = dxm * a1 ** (ALx1 + ALx2 - i)
    for i in range(ALx2 - 1, -1, -1):
        dx[i] = dxm * a1 ** ALx1 * a2 ** (ALx2 - i)
    for i in range(Nx + AL, Nx + AL + ARx1):
        dx[i] = dxm * a1 ** (i - AL - Nx + 1)
    for i in range(Nx + AL + ARx1, L):
        dx[i] = dxm * a1 ** ARx1 * a2 ** (i - Nx - AL - ARx1 + 1)
    Ay = Ay2 + Ay1
    dy = np.zeros(M)
    dy[Ay:Ay + Ny] = dym
    for j in range(Ay - 1, Ay2 - 1, -1):
        dy[j] = dy[j + 1] * a1
    for j in range(Ay2 - 1, -1, -1):
        dy[j] = dy[j + 1] * a2
    for j in range(Ny + Ay, Ny + Ay2 + 2 * Ay1):
        dy[j] = dy[j - 1] * a1
    for j in range(Ny + Ay2 + 2 * Ay1, M):
        dy[j] = dy[j - 1] * a2
    dz = np.zeros(N)
    dz[:Nz] = dzm
    for k in range(Nz, Nz + Az1):
        dz[k] = dz[k - 1] * a1
    for k in range(Nz + Az1, N):
        dz[k] = dz[k - 1] * a2
    x0, y0, z0 = c.get("origin", (0.0, 0.0, 0.0))

    def centres(d, n_core, lead, o):
        n = len(d)
        X = np.zeros(n)
        if n_core % 2 == 0:
            nc = n_core // 2 + lead
            X[nc] = 0.5 * d[nc] + o
        else:
            nc = (n_core - 1) // 2 + lead
            X[nc] = o
        for i in range(nc + 1, n):
            X[i] = X[i - 1] + 0.5 * d[i - 1] + 0.5 * d[i]
        for i in range(nc - 1, -1, -1):
            X[i] = X[i + 1] - 0.5 * d[i + 1] - 0.5 * d[i]
        return X

    X = centres(dx, Nx, AL, x0)
    Y = centres(dy, Ny, Ay, y0)
    Z = np.zeros(N)
    Z[0] = 0.5 * dz[0] + z0
    for k in range(1, N):
        Z[k] = Z[k - 1] + 0.5 * dz[k - 1] + 0.5 * dz[k]
    return dict(L=L, M=M, N=N, dx=dx, dy=dy, dz=dz, X=X, Y=Y, Z=Z)


def plane_size(c):
    """Size L1 x M1 of the uniform continuation plane (ModelingSetup.cpp:190-192)."""
    g = grid_axes(c)
    ALx2, ALx1, Nx, ARx1, ARx2 = c["xsplit"]
    Ay2, Ay1, Ny = c["ysplit"]
    dxm, dym, _ = c["dmin"]
    X, Y, dx, dy, L = g["X"], g["Y"], g["dx"], g["dy"], g["L"]
    AL = ALx1 + ALx2
    AR0 = L - ARx1 - ARx2
    anl = math.ceil((X[AL - 1] - X[0] + dx[AL - 1] / 2 + dx[0] / 2) / dxm)
    anr = math.ceil((X[L - 1] - X[AR0] + dx[L - 1] / 2 + dx[AR0] / 2) / dxm)
    Ay = Ay1 + Ay2
    any_ = math.ceil((Y[Ay - 1] - Y[0] + dy[Ay - 1] / 2 + dy[0] / 2) / dym)
    return anl + anr + Nx, 2 * any_ + Ny


# --------------------------------------------------------------------------- writers


def _fmt(v):
    return repr(float(v))


def write_case(c, directory):
    """Write the four input files of case ``c`` into ``directory``; returns the directory."""
    os.makedirs(directory, exist_ok=True)
    g = grid_axes(c)
    with open(os.path.join(directory, "FDTD_setup.in"), "w") as f:
        f.write(f"{_fmt(c['sfa1'])} {_fmt(c['sfa2'])}\n")
        f.write(f"{int(c['n1'])} {_fmt(c['sita_t'])}\n")
        f.write(" ".join(_fmt(v) for v in c.get("origin", (0.0, 0.0, 0.0))) + "\n")
        f.write(" ".join(_fmt(v) for v in c["dmin"]) + "\n")
        f.write(f"{_fmt(c['arg1'])} {_fmt(c['arg2'])}\n")
        f.write(" ".join(str(int(v)) for v in c["xsplit"]) + "\n")
        f.write(" ".join(str(int(v)) for v in c["ysplit"]) + "\n")
        f.write(" ".join(str(int(v)) for v in c["zsplit"]) + "\n")
    con = conductivity(c, g)
    assert con.shape == (g["N"], g["M"], g["L"])
    np.ascontiguousarray(con, dtype="<f8").tofile(os.path.join(directory, "Cond.bin"))
    rx = c["receivers"]
    with open(os.path.join(directory, "Receiver.in"), "w") as f:
        f.write(f"{_fmt(c['T0'])} {_fmt(c['Tn'])}\n")
        f.write(f"{int(c['Nt'])} {int(c['islog'])}\n")
        f.write(" ".join(str(int(v)) for v in c["comps"]) + "\n")
        f.write(f"{len(rx)}\n")
        for i, (x, y, z) in enumerate(rx):
            f.write(f"{i + 1} {_fmt(x)} {_fmt(y)} {_fmt(z)}\n")
    with open(os.path.join(directory, "Transmitter.in"), "w") as f:
        f.write(f"{len(c['transmitters'])}\n")
        for i, t in enumerate(c["transmitters"]):
            ids = t.get("rx", list(range(1, len(rx) + 1)))
            parts = [str(i + 1), str(int(t["ort"])), _fmt(t["len"]), _fmt(t["x"]), _fmt(t["y"]), _fmt(t["z"])]
            if t["ort"] >= 4:
                parts += [_fmt(t["azi"]), _fmt(t["dip"])]
            if t["ort"] == 5:
                parts += [_fmt(t["len1"]), _fmt(t["x1"]), _fmt(t["y1"]), _fmt(t["z1"]), _fmt(t["azi1"]),
                          _fmt(t["dip1"])]
            parts += [str(len(ids))] + [str(v) for v in ids]
            f.write(" ".join(parts) + "\n")
    return directory


# --------------------------------------------------------------------------- models


def _smooth_noise(shape, sigma_cells, seed):
    """Gaussian-filtered white noise with unit standard deviation (seeded)."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(shape)
    out = w
    for ax, s in enumerate(sigma_cells):
        if s <= 0:
            continue
        r = int(math.ceil(3 * s))
        t = np.arange(-r, r + 1)
        k = np.exp(-0.5 * (t / s) ** 2)
        k /= k.sum()
        out = np.apply_along_axis(lambda v: np.convolve(np.pad(v, r, mode="wrap"), k, mode="valid"), ax, out)
    sd = out.std()
    return out / sd if sd > 0 else out


def conductivity(c, g=None):
    """Conductivity array [N][M][L] (S/m) for case ``c``."""
    g = g or grid_axes(c)
    N, M, L = g["N"], g["M"], g["L"]
    Zc, Yc, Xc = g["Z"], g["Y"], g["X"]
    m = c["model"]
    kind = m["kind"]
    if kind == "uniform":
        return np.full((N, M, L), float(m["sigma"]))
    if kind == "random":
        rng = np.random.default_rng(m.get("seed", 0))
        lo, hi = m.get("range", (0.1, 4.0))
        return np.exp(rng.uniform(np.log(lo), np.log(hi), size=(N, M, L)))
    if kind == "layered":  # horizontal layers [(z_top, sigma), ...] below z = 0, plus blocks
        con = np.empty((N, M, L))
        zc = Zc[:, None, None] * np.ones((1, M, L))
        con[:] = m["layers"][0][1]
        for (ztop, s) in m["layers"]:
            con[zc >= ztop] = s
        for b in m.get("blocks", []):
            xs, ys, zs, s = b
            sel = ((Xc[None, None, :] >= xs[0]) & (Xc[None, None, :] < xs[1]) &
                   (Yc[None, :, None] >= ys[0]) & (Yc[None, :, None] < ys[1]) &
                   (Zc[:, None, None] >= zs[0]) & (Zc[:, None, None] < zs[1]))
            con[sel] = s
        return con
    if kind == "marine":
        con = np.empty((N, M, L))
        zc = Zc[:, None, None] * np.ones((1, M, L))
        con[:] = m["sediment"]
        con[zc < m["water_depth"]] = m["water"]
        for (ztop, zbot, s) in m.get("layers", []):
            con[(zc >= ztop) & (zc < zbot)] = s
        if "perturb" in m:
            p = m["perturb"]
            sig = [p["corr"] / g["dz"].min(), p["corr"] / g["dy"].min(), p["corr"] / g["dx"].min()]
            noise = _smooth_noise((N, M, L), sig, p["seed"])
            sed = zc >= m["water_depth"]
            con[sed] = con[sed] * 10.0 ** (p["sigma_log10"] * noise[sed])
        for b in m.get("blocks", []):
            xs, ys, zs, s = b
            sel = ((Xc[None, None, :] >= xs[0]) & (Xc[None, None, :] < xs[1]) &
                   (Yc[None, :, None] >= ys[0]) & (Yc[None, :, None] < ys[1]) &
                   (Zc[:, None, None] >= zs[0]) & (Zc[:, None, None] < zs[1]))
            con[sel] = s
        return con
    raise ValueError(f"unknown model kind {kind}")


# --------------------------------------------------------------------------- named cases


def _base(**kw):
    c = dict(sfa1=1.5, sfa2=2.0, n1=200, sita_t=1e-5, origin=(0.0, 0.0, 0.0), comps=(1, 1, 0, 1, 1, 1), islog=1)
    c.update(kw)
    return c


CASES = {
    # small grids for the parity tests (the oracle finishes these in seconds)
    "tiny": _base(
        dmin=(50.0, 50.0, 50.0), arg1=1.2, arg2=1.3, xsplit=(2, 5, 12, 5, 2), ysplit=(2, 5, 10), zsplit=(2, 6, 8),
        n1=200, sita_t=1e-4, T0=2e-3, Tn=2e-2, Nt=12, comps=(1, 1, 1, 1, 1, 1),
        model=dict(kind="random", seed=7, range=(0.05, 3.0)),
        receivers=[(-75.0 + 50 * i, 25.0 * (i % 3) - 25.0, 0.0 if i % 2 == 0 else 60.0) for i in range(5)],
        transmitters=[dict(ort=1, len=100.0, x=-10.0, y=5.0, z=20.0)],
    ),
    "small": _base(
        dmin=(40.0, 40.0, 40.0), arg1=1.15, arg2=1.25, xsplit=(3, 8, 20, 10, 3), ysplit=(3, 8, 16), zsplit=(3, 10, 14),
        n1=200, sita_t=1e-4, T0=1e-3, Tn=5e-2, Nt=24,
        model=dict(kind="marine", water=3.2, sediment=1.0, water_depth=200.0, layers=[(400.0, 480.0, 0.01)],
                   perturb=dict(sigma_log10=0.2, corr=120.0, seed=42)),
        receivers=[(-120.0 + 80.0 * i, 20.0, 200.0) for i in range(6)],
        transmitters=[dict(ort=1, len=80.0, x=-200.0, y=0.0, z=150.0)],
    ),
    # several transmitter orientations on the tiny grid (ort 1..5 of LoadRxTxPos.cpp)
    "txvar": _base(
        dmin=(50.0, 50.0, 50.0), arg1=1.2, arg2=1.3, xsplit=(2, 5, 12, 5, 2), ysplit=(2, 5, 10), zsplit=(2, 6, 8),
        n1=200, sita_t=1e-4, T0=2e-3, Tn=2e-2, Nt=12, comps=(1, 1, 1, 1, 1, 1),
        model=dict(kind="random", seed=11, range=(0.05, 3.0)),
        receivers=[(-75.0 + 50 * i, 25.0 * (i % 3) - 25.0, 0.0 if i % 2 == 0 else 60.0) for i in range(5)],
        transmitters=[dict(ort=1, len=100.0, x=-10.0, y=5.0, z=20.0, rx=[1, 3, 5]),
                      dict(ort=2, len=120.0, x=30.0, y=-20.0, z=80.0, rx=[2, 4]),
                      dict(ort=3, len=90.0, x=-40.0, y=40.0, z=150.0),
                      dict(ort=4, len=150.0, x=10.0, y=10.0, z=100.0, azi=30.0, dip=20.0, rx=[5, 4, 3, 2, 1]),
                      dict(ort=4, len=120.0, x=0.0, y=0.0, z=60.0, azi=90.0, dip=0.0, rx=[1]),
                      dict(ort=5, len=100.0, x=-30.0, y=0.0, z=120.0, azi=45.0, dip=10.0,
                           len1=80.0, x1=60.0, y1=-30.0, z1=60.0, azi1=-20.0, dip1=5.0)],
    ),
    # the reference's shipped example grid (FDTD_setup.in of the reference tree), synthetic 1 S/m model
    "example": _base(
        dmin=(50.0, 50.0, 50.0), arg1=1.1, arg2=1.2, xsplit=(10, 40, 120, 40, 10), ysplit=(10, 40, 100),
        zsplit=(10, 40, 60), n1=200, sita_t=1e-3, sfa1=2.0, sfa2=2.0, T0=0.01, Tn=10.0, Nt=100,
        comps=(1, 1, 0, 1, 1, 1), model=dict(kind="uniform", sigma=1.0),
        receivers=[(1500.0 + 500.0 * i, 0.0, 1000.0) for i in range(5)],
        transmitters=[dict(ort=1, len=200.0, x=0.0, y=0.0, z=600.0)],
    ),
    # a grid three sweep tiles wide (142 = 2 x 64 + 14: a partial last x-tile) and five
    # tile rows high (36 = 4 x 8 + 4), random conductivity, transmitters that cross the
    # tile boundaries at i = 64 (x-directed) and j = 16 (y-directed), receivers spread
    # over every tile; its 192 x 76 continuation plane keeps the oracle fast
    "wide_142x36x25": _base(
        dmin=(40.0, 40.0, 40.0), arg1=1.15, arg2=1.25, xsplit=(3, 8, 118, 10, 3), ysplit=(3, 8, 14),
        zsplit=(3, 8, 14), n1=200, sita_t=1e-4, T0=1e-3, Tn=5e-2, Nt=24, comps=(1, 1, 1, 1, 1, 1),
        model=dict(kind="random", seed=23, range=(0.05, 3.0)),
        receivers=[(-2200.0 + 300.0 * i, 40.0 * (i % 4) - 60.0, 0.0 if i % 3 else 120.0) for i in range(16)],
        transmitters=[dict(ort=1, len=200.0, x=-240.0, y=20.0, z=60.0),
                      dict(ort=2, len=160.0, x=1100.0, y=-70.0, z=100.0),
                      dict(ort=4, len=200.0, x=2330.0, y=-40.0, z=140.0, azi=35.0, dip=25.0)],
    ),
    # survey config 1: homogeneous 1 S/m half-space, 64 x 64 x 48, 25 m, growth 1.15
    "halfspace_64x64x48": _base(
        dmin=(25.0, 25.0, 25.0), arg1=1.15, arg2=1.15, xsplit=(0, 12, 24, 28, 0), ysplit=(0, 20, 24),
        zsplit=(0, 28, 20), n1=200, sita_t=1e-5, sfa1=1.5, sfa2=2.0, T0=1e-4, Tn=1.0, Nt=61,
        comps=(1, 1, 0, 0, 1, 1), model=dict(kind="uniform", sigma=1.0),
        receivers=[(500.0 + 250.0 * i, 0.0, 0.0) for i in range(15)],
        transmitters=[dict(ort=1, len=25.0, x=0.0, y=0.0, z=0.0)],
    ),
    # the same half-space survey refined two-fold: 12.5 m core cells and growth 1.075, so
    # every cell near the receivers is about half its size in halfspace_64x64x48 (a 2 km
    # offset sits in 136 m cells instead of 269 m), over about the same extents; 960 x 576 plane
    "halfspace_refined_133x130x95": _base(
        dmin=(12.5, 12.5, 12.5), arg1=1.075, arg2=1.075, xsplit=(0, 29, 48, 56, 0), ysplit=(0, 41, 48),
        zsplit=(0, 55, 40), n1=200, sita_t=1e-5, sfa1=1.5, sfa2=2.0, T0=1e-4, Tn=1.0, Nt=61,
        comps=(1, 1, 0, 0, 1, 1), model=dict(kind="uniform", sigma=1.0),
        receivers=[(500.0 + 250.0 * i, 0.0, 0.0) for i in range(15)],
        transmitters=[dict(ort=1, len=25.0, x=0.0, y=0.0, z=0.0)],
    ),
    # uniform 1 S/m half-space fine enough for the closed-form check: 12.5 m core
    # cells, growth 1.2, x-directed 25 m wire at the surface, inline receivers
    # at 250-1000 m on the surface
    "halfspace": _base(
        dmin=(12.5, 12.5, 12.5), arg1=1.2, arg2=1.2, xsplit=(0, 20, 120, 20, 0), ysplit=(0, 20, 16),
        zsplit=(0, 20, 20), n1=200, sita_t=1e-5, sfa1=1.5, sfa2=2.0, T0=1e-3, Tn=0.3, Nt=41,
        comps=(1, 1, 0, 0, 1, 1), model=dict(kind="uniform", sigma=1.0),
        receivers=[(250.0 * (i + 1), 0.0, 0.0) for i in range(4)],
        transmitters=[dict(ort=1, len=25.0, x=0.0, y=0.0, z=0.0)],
    ),
    # survey config 2: 1-D marine model, 128 x 128 x 96 at 20 m
    "marine1d_128x128x96": _base(
        dmin=(20.0, 20.0, 20.0), arg1=1.06, arg2=1.15, xsplit=(6, 14, 48, 50, 10), ysplit=(6, 14, 88),
        zsplit=(10, 30, 56), n1=200, sita_t=1e-4, sfa1=2.0, sfa2=2.0, T0=1e-3, Tn=10.0, Nt=81,
        comps=(1, 1, 0, 1, 1, 1),
        model=dict(kind="marine", water=3.2, sediment=1.0, water_depth=1000.0, layers=[(2000.0, 2100.0, 0.01)]),
        receivers=[(250.0 + 250.0 * i, 0.0, 1000.0) for i in range(40)],
        transmitters=[dict(ort=1, len=40.0, x=0.0, y=0.0, z=950.0)],
    ),
    # survey config 3: 3-D marine model, 256 x 256 x 160 at 25 m
    "marine3d_256x256x160": _base(
        dmin=(25.0, 25.0, 25.0), arg1=1.08, arg2=1.08, xsplit=(0, 40, 176, 40, 0), ysplit=(0, 40, 176),
        zsplit=(0, 60, 100), n1=200, sita_t=1e-4, sfa1=2.0, sfa2=2.0, T0=1e-3, Tn=10.0, Nt=81,
        comps=(1, 1, 0, 1, 1, 1),
        model=dict(kind="marine", water=3.2, sediment=1.0, water_depth=1000.0,
                   perturb=dict(sigma_log10=0.2, corr=200.0, seed=42),
                   blocks=[((-2000.0, 2000.0), (-2000.0, 2000.0), (2000.0, 2100.0), 0.01)]),
        receivers=[(-5000.0 + 500.0 * i, -5000.0 + 500.0 * j, 1000.0) for j in range(21) for i in range(21)],
        transmitters=[dict(ort=1, len=50.0, x=0.0, y=0.0, z=950.0)],
    ),
    # the 3-D marine survey on the same 256 x 256 x 160 grid with 35-cell (not 40-cell) boundary
    # strips: 187 uniform continuation points per strip instead of 280, below the 256 points
    # one block of the reference's strip kernels covers (see the oracle's notes on
    # SplineGridConvIR2R.cu:180-498); 560 x 560 plane
    "marine3d_strip35_256x256x160": _base(
        dmin=(25.0, 25.0, 25.0), arg1=1.08, arg2=1.08, xsplit=(0, 35, 186, 35, 0), ysplit=(0, 35, 186),
        zsplit=(0, 60, 100), n1=200, sita_t=1e-4, sfa1=2.0, sfa2=2.0, T0=1e-3, Tn=10.0, Nt=81,
        comps=(1, 1, 0, 1, 1, 1),
        model=dict(kind="marine", water=3.2, sediment=1.0, water_depth=1000.0,
                   perturb=dict(sigma_log10=0.2, corr=200.0, seed=42),
                   blocks=[((-2000.0, 2000.0), (-2000.0, 2000.0), (2000.0, 2100.0), 0.01)]),
        receivers=[(-5000.0 + 500.0 * i, -5000.0 + 500.0 * j, 1000.0) for j in range(21) for i in range(21)],
        transmitters=[dict(ort=1, len=50.0, x=0.0, y=0.0, z=950.0)],
    ),
}


def batch_case(seed, size=((96, 192), (96, 192), (96, 128)), tn=(1.0,)):
    """One survey of the batched workload, drawn from ``seed``.

    Grid uniform in [96, 192] x [96, 192] x [96, 128] cells at 25 m (20-cell
    boundary strips growing by 1.08 on each lateral side and at the bottom),
    a background of 1-3 horizontal layers with resistivities 0.3-5 ohm-m, a
    20-200 ohm-m resistive block, an x-directed transmitter placed along a line
    through the core, 40 inline receivers, time window 1e-3 s to one of `tn`.
    """
    rng = np.random.default_rng(seed)
    L, M, N = (int(rng.integers(a, b + 1)) for a, b in size)
    strip, dmin = 20, 25.0
    nx, ny, nz = L - 2 * strip, M - 2 * strip, N - strip
    half_x, depth = 0.5 * nx * dmin, nz * dmin
    nl = int(rng.integers(1, 4))
    tops = [0.0] + sorted(float(z) for z in rng.uniform(0.15 * depth, 0.8 * depth, nl - 1))
    layers = [(z, 1.0 / float(rng.uniform(0.3, 5.0))) for z in tops]
    bx = float(rng.uniform(0.15, 0.35)) * 2 * half_x
    bz0 = float(rng.uniform(0.4, 0.7)) * depth
    block = ((-0.5 * bx, 0.5 * bx), (-0.5 * bx, 0.5 * bx), (bz0, bz0 + 4 * dmin), 1.0 / float(rng.uniform(20.0, 200.0)))
    ztx = round(0.3 * depth / dmin) * dmin + 0.5 * dmin
    xtx = float(rng.uniform(-0.5, 0.5)) * half_x
    xr = np.linspace(-0.8 * half_x, 0.8 * half_x, 40)
    return _base(
        dmin=(dmin, dmin, dmin), arg1=1.08, arg2=1.08, xsplit=(0, strip, nx, strip, 0), ysplit=(0, strip, ny),
        zsplit=(0, strip, nz), n1=200, sita_t=1e-4, sfa1=2.0, sfa2=2.0, T0=1e-3, Tn=float(rng.choice(tn)), Nt=41,
        comps=(1, 1, 0, 1, 1, 1), model=dict(kind="layered", layers=layers, blocks=[block]),
        receivers=[(float(x), 0.0, ztx + dmin) for x in xr],
        transmitters=[dict(ort=1, len=2 * dmin, x=xtx, y=0.0, z=ztx)],
    )


def memory_case(c):
    """The survey of case ``c`` as the (model, survey) values of the in-memory open
    (api.memory_records / tcsem_open): the same numbers write_case puts in the four files."""
    g = grid_axes(c)
    ALx2, ALx1, Nx, ARx1, ARx2 = c["xsplit"]
    Ay2, Ay1, Ny = c["ysplit"]
    Az2, Az1, Nz = c["zsplit"]
    x0, y0, z0 = c.get("origin", (0.0, 0.0, 0.0))
    model = dict(sfa1=c["sfa1"], sfa2=c["sfa2"], n1=int(c["n1"]), sita_t=c["sita_t"], x0=x0, y0=y0, z0=z0,
                 dxmin=c["dmin"][0], dymin=c["dmin"][1], dzmin=c["dmin"][2], arg1=c["arg1"], arg2=c["arg2"],
                 ALx2=ALx2, ALx1=ALx1, Nx=Nx, ARx1=ARx1, ARx2=ARx2, Ay2=Ay2, Ay1=Ay1, Ny=Ny, Az2=Az2, Az1=Az1, Nz=Nz,
                 con=conductivity(c, g))
    rx = c["receivers"]
    tx = []
    for t in c["transmitters"]:
        d = dict(ort=int(t["ort"]), len=t["len"], x=t["x"], y=t["y"], z=t["z"],
                 rx=list(t.get("rx", range(1, len(rx) + 1))))
        if t["ort"] >= 4:
            d.update(azi=t["azi"], dip=t["dip"])
        if t["ort"] == 5:
            d.update(len1=t["len1"], x1=t["x1"], y1=t["y1"], z1=t["z1"], azi1=t["azi1"], dip1=t["dip1"])
        tx.append(d)
    survey = dict(T0=c["T0"], Tn=c["Tn"], Nt=int(c["Nt"]), IsLog=int(c["islog"]), comps=list(c["comps"]),
                  rx_xyz=np.array(rx, dtype=np.float64), tx=tx)
    return model, survey


def case(name, **overrides):
    c = copy.deepcopy(CASES[name])
    c.update(overrides)
    return c


def steps_estimate(c):
    """Number of steps of the reference's Delta-t rule up to Tn (main.cu:150-165), for sizing."""
    nsrc = c["n1"] // 2
    mindx = min(c["dmin"])
    t = 6 * c["sita_t"]
    dt1 = 0.15 * c["sfa1"] * math.sqrt(MU0 * t * 0.1 / 8) * mindx
    n = 2 * nsrc
    while t <= c["Tn"]:
        dt2 = min(0.15 * c["sfa1"] * math.sqrt(MU0 * t * 0.1 / 8) * mindx, 1.2 * dt1)
        n += 1
        t += dt2
        dt1 = dt2
    return n + 1
