"""The oracle's boundary operator: linear in the Bz plane, and the FFT it uses agrees with numpy."""
import numpy as np
import pytest


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_oracle_continuation_is_linear(name, case_dir):
    from oracle.oracle import Oracle

    o = Oracle(case_dir(name))
    rng = np.random.default_rng(3)
    shp = o.field_shape("Bz")
    a, b = rng.standard_normal(shp), rng.standard_normal(shp)
    outs = []
    for z in (a, b, 2.0 * a - 3.0 * b):
        o.zero()
        o.set("Bz", z)
        o.upcontinuation()
        outs.append((o.get("BxAir"), o.get("ByAir")))
    for q in range(2):
        lin = 2 * outs[0][q] - 3 * outs[1][q]
        np.testing.assert_allclose(outs[2][q], lin, rtol=0, atol=1e-11 * np.abs(lin).max())


@pytest.mark.parametrize("name", ["tiny", "small", "halfspace_64x64x48"])
def test_oracle_spline_remap_keeps_core_and_is_exact_on_linear_data(name, case_dir):
    """The natural spline reproduces linear data in the strips (the end-derivative extrapolation too)."""
    from oracle.oracle import Oracle

    o = Oracle(case_dir(name))
    X, Y = o.darray("X"), o.darray("Y")
    Xn, Yn = o.darray("Xn"), o.darray("Yn")
    bz = np.zeros(o.field_shape("Bz"))
    bz[0] = 3.0 + 0.002 * X[None, :] - 0.001 * Y[:, None]
    o.zero()
    o.set("Bz", bz)
    o.spline_remap()
    got = o.get("BzAir")
    exp = 3.0 + 0.002 * Xn[None, :] - 0.001 * Yn[:, None]
    np.testing.assert_allclose(got, exp, rtol=1e-9, atol=1e-9)


def test_padded_continuation_of_a_central_blob():
    """The oracle's padded-plane continuation (not the reference's arithmetic) moves a smooth
    field in the middle of the plane by a few percent at most: the padding changes the
    periodic images and the DC bin, not the local field."""
    import tempfile

    from oracle.oracle import Oracle, build
    from tcsem_fdtd_gb300 import inputs

    build()
    d = tempfile.mkdtemp()
    inputs.write_case(inputs.case("small"), d)
    o = Oracle(d)
    X, Y = np.meshgrid(o.darray("X"), o.darray("Y"))
    bz = np.zeros(o.field_shape("Bz"))
    bz[0] = np.exp(-(X ** 2 + Y ** 2) / (2 * 150.0 ** 2))
    out = []
    for padded in (False, True):
        o.set("Bz", bz)
        if padded:
            o.set_padded_plane(1)
            o.upcontinuation_padded()
        else:
            o.upcontinuation()
        out.append((o.get("BxAir").copy(), o.get("ByAir").copy()))
    for a, b in zip(*out):
        assert np.all(np.isfinite(b))
        assert np.abs(a - b).max() / np.abs(a).max() < 0.05
