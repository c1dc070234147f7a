"""The learned-closure experiment's numpy side (tlbm_gb300/closure.py) on fields with known
answers: the strain rate, the least-squares sub-grid eddy viscosity, the features, the
spectrum and profile metrics, the inlet fields and the normalisation.  No GPU."""

import numpy as np
import pytest

from tlbm_gb300 import closure as CL


def shear_field(nz=4, ny=16, nx=8):
    y = np.arange(ny)[None, :, None] * np.ones((nz, ny, nx))
    ux = np.sin(2 * np.pi * y / ny)
    zero = np.zeros_like(ux)
    return ux, zero, zero.copy(), y


def test_strain_of_a_periodic_shear():
    ux, uy, uz, y = shear_field()
    ny = ux.shape[1]
    S = CL.strain(ux, uy, uz)
    # central difference of sin(k y): cos(k y) sin(k)
    want_xy = 0.5 * np.cos(2 * np.pi * y / ny) * np.sin(2 * np.pi / ny)
    assert np.allclose(S[3], want_xy, atol=1e-15)
    for k in (0, 1, 2, 4, 5):
        assert np.abs(S[k]).max() == 0.0


@pytest.mark.parametrize("nu0", [3e-4, -3e-4])
def test_sgs_eddy_viscosity_recovers_a_known_viscosity(nu0):
    """A sub-grid stress tau = -2 nu0 S gives back nu_t = nu0 where the strain is non-zero;
    a negative nu0 is clipped to 0, and nu_cap caps it."""
    ux, uy, uz, _ = shear_field()
    S = CL.strain(ux, uy, uz)
    F = {"ux": ux, "uy": uy, "uz": uz, "rho": np.ones_like(ux),
         "uxux": ux * ux, "uyuy": uy * uy, "uzuz": uz * uz,
         "uxuy": ux * uy - 2 * nu0 * S[3], "uxuz": ux * uz, "uyuz": uy * uz}
    nut, S2 = CL.sgs_eddy_viscosity(F, nu_cap=1.0)
    strained = np.abs(S[3]) > 1e-6
    assert strained.any()
    assert np.allclose(nut[strained], max(nu0, 0.0), rtol=1e-9, atol=1e-15)
    assert np.all(nut[~strained] == 0.0)
    capped, _ = CL.sgs_eddy_viscosity(F, nu_cap=1e-4)
    assert capped.max() <= 1e-4


def test_raw_features_are_the_stress_a_coarse_node_sees():
    ux, uy, uz, _ = shear_field()
    S = CL.strain(ux, uy, uz)
    rho = np.full_like(ux, 1.01)
    nu, nut = 0.01, np.full_like(ux, 0.002)
    x = CL.raw_features({"rho": rho}, S, nu, nut)
    tau = 3 * (nu + 0.002) + 0.5
    assert x.shape == (ux.size, 8)
    assert np.allclose(x[:, 3], (-2 * 1.01 * CL.CS2 * tau * S[3]).reshape(-1))
    assert np.allclose(x[:, 6], 0.01)
    assert np.allclose(x[:, 7], np.sqrt(2) * np.abs(x[:, 3]))


def test_spectrum_puts_a_single_mode_in_its_bin():
    nz, ny, nx = 3, 16, 32
    x = np.arange(nx)[None, None, :] * np.ones((nz, ny, nx))
    uz = 0.2 + np.cos(2 * np.pi * 3 * x / nx)
    e = CL.spectrum(uz, [0, 2])
    assert np.isclose(e[3], 0.5)
    assert np.isclose(e.sum(), 0.5)


def test_mean_profile_and_rel_l2():
    nd = np.zeros((5, 4, 3), np.int32)
    uz = np.arange(5, dtype=np.float64)[:, None, None] * np.ones((5, 4, 3))
    assert np.array_equal(CL.mean_profile(uz.reshape(-1), nd), np.arange(5.0))
    assert CL.rel_l2(np.array([1.0, 2.0]), np.array([1.0, 2.0])) == 0.0
    assert np.isclose(CL.rel_l2(np.array([2.0, 0.0]), np.array([1.0, 0.0])), 1.0)


def test_inlet_fields():
    j = CL.jet_profile(8, 32, factor=2, ratio=0.5)
    assert j.shape == (64, 16)
    col = j[:, 0]
    assert np.allclose(col, col[::-1], atol=1e-12)  # symmetric about the middle of the period
    assert col.max() <= 0.5 and col[len(col) // 2] > 0.49 and col[0] < 0.01
    n1 = CL.inlet_noise(8, 6, factor=1, seed=4)
    n2 = CL.inlet_noise(8, 6, factor=1, seed=4)
    assert n1.shape == (6, 8) and np.array_equal(n1, n2)
    assert abs(n1.mean()) < 1e-12 and np.isclose(n1.std(), 1.0)
    u = CL.inlet_velocity(8, 6, 1, 0.05, 0.01, 0.5, 4)
    assert np.all(u > 0.04) and np.all(u < 0.08)


def test_normalise_and_dataset_drop_non_finite_cells():
    rng = np.random.default_rng(0)
    raw = rng.normal(3.0, 2.0, size=(1000, 8))
    t = rng.uniform(0, 1e-3, size=1000)
    shift, scale, out_scale = CL.normalise(raw, t)
    x = (raw - shift) * scale
    assert np.allclose(x.mean(0), 0.0, atol=1e-6) and np.allclose(x.std(0), 1.0, atol=1e-5)
    assert np.isclose(out_scale, t.std())
    ux, uy, uz, _ = shear_field()
    F = {"ux": ux, "uy": uy, "uz": uz, "rho": np.ones_like(ux),
         "uxux": ux * ux, "uyuy": uy * uy, "uzuz": uz * uz,
         "uxuy": ux * uy, "uxuz": ux * uz, "uyuz": uy * uz}
    F["rho"][0, 0, 0] = np.nan
    feats, targets = CL.build_dataset({0: F}, 0.01, 1.0)
    assert len(feats) == ux.size - 1 and len(targets) == ux.size - 1
    assert np.isfinite(feats).all()
