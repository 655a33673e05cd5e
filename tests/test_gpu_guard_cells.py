"""Guard cells stay untouched.

The device arrays pad every component to one geometry (x from -4, one row
below 0 and above M-1, one plane above 0 and below N-1; see kernels.cuh); the
stencils read the cells outside a component's extent as the zero boundary, so
no kernel may ever write them.  A saved run state (tcsem_save_state) holds the
raw padded arrays of the current fields: after steps in both precisions and
step orders, every cell outside each component's extent -- and, for Bx and By,
outside the air plane the boundary writes at k = -1 -- must still be exactly 0.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KMAX = 16  # chunk boundaries stored in the state header: KMAX + 1 (kMaxChunks of kernels.cuh)


def read_state(path):
    raw = open(path, "rb").read()
    assert raw[:7] == b"TCSEMST"
    ints = np.frombuffer(raw, dtype="<i4", count=8, offset=8)  # version tsize L M N itx cur nch
    off = 8 + 4 * 8 + 4 * (KMAX + 1)
    off += (-off) % 8
    step, field_bytes, tot_bytes, ef0_bytes, efs_bytes = np.frombuffer(raw, dtype="<i8", count=5, offset=off)
    off += 5 * 8
    assert int(ints[0]) == 2  # version 2: L1 M1 padded_plane fix_dual_bipole (int32), nsteps (int64) follow
    off += 4 * 4 + 8
    assert len(raw) == off + 6 * int(field_bytes) + int(tot_bytes) + int(ef0_bytes) + int(efs_bytes)
    tsize, L, M, N = int(ints[1]), int(ints[2]), int(ints[3]), int(ints[4])
    dt = "<f8" if tsize == 8 else "<f4"
    XP = (L + 6 + 31) // 32 * 32
    arrays = []
    for _ in range(6):
        a = np.frombuffer(raw, dtype=dt, count=int(field_bytes) // tsize, offset=off)
        arrays.append(a.reshape(N + 2, M + 2, XP))
        off += int(field_bytes)
    return (L, M, N), arrays, int(step)


def extent_mask(shape, L, M, N, comp):
    """Padded cells a component may hold: its reference extent, and the air plane of Bx/By."""
    ext = {0: (L, M + 1, N + 1), 1: (L + 1, M, N + 1), 2: (L + 1, M + 1, N), 3: (L + 1, M, N), 4: (L, M + 1, N),
           5: (L, M, N + 1)}[comp]
    mask = np.zeros(shape, dtype=bool)
    nx, ny, nz = ext
    mask[1:1 + nz, 1:1 + ny, 4:4 + nx] = True  # k >= 0, j >= 0, i >= 0
    if comp == 3:
        mask[0, 1:1 + M, 4:4 + L + 1] = True  # BxAir
    if comp == 4:
        mask[0, 1:1 + M + 1, 4:4 + L] = True  # ByAir
    return mask


@pytest.fixture(scope="module")
def built():
    from tcsem_fdtd_gb300 import build

    build.build()
    return True


@pytest.mark.parametrize("precision,zchunks,serial", [(32, 0, False), (64, 4, True), (32, 5, False)])
@pytest.mark.parametrize("name", ["small", "txvar"])
def test_guard_cells_stay_zero(built, case_dir, tmp_path, name, precision, zchunks, serial):
    from tcsem_fdtd_gb300 import Simulation

    path = tmp_path / "state.bin"
    with Simulation(case_dir(name), precision=precision, zchunks=zchunks, serial_boundary=serial) as sim:
        sim.begin(0)
        sim.advance(min(301, sim.info["nsteps"]))  # through the source window
        sim.save_state(path)
    (L, M, N), arrays, step = read_state(path)
    assert step > 0
    for comp, a in enumerate(arrays):
        mask = extent_mask(a.shape, L, M, N, comp)
        stray = np.flatnonzero(a[~mask] != 0)
        assert stray.size == 0, (comp, stray.size)
        assert np.abs(a[mask]).max() > 0  # the fields did move
