"""Learned closure on the GPU: training gradients against the CPU oracle, training, inference
inside the collide kernel, the box filter and the inlet profile it is trained with."""

import numpy as np
import pytest

import mlp_oracle as M
import tlbm_gb300 as T
from tlbm_gb300 import build as B
from tlbm_gb300 import closure as CL
from tlbm_gb300 import geometry as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    B.build()
    T.library()


def data(n=3000, seed=2):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 8)).astype(np.float32)
    t = (0.5 * np.tanh(X[:, 0] - 0.5 * X[:, 3]) + 0.2 * X[:, 7] ** 2 - 0.1).astype(np.float32)
    return X, t


def test_gradient_matches_oracle():
    X, t = data()
    p = M.init_params(7)
    tr = T.MlpTrainer(X, t, seed=1)
    tr.set_params(p)
    loss, g = tr.loss_grad()
    loss_o, g_o, _ = M.forward_backward(p, X, t)
    assert abs(loss - loss_o) <= 1e-3 * abs(loss_o)
    err = np.linalg.norm(g - g_o) / np.linalg.norm(g_o)
    print("gradient relative L2 error vs oracle: %.2e" % err)
    # the kernels and the oracle round the same values to BF16; what differs is FP32 against
    # FP64 accumulation and the special-function tanh (relative error below 2^-10.9), which
    # moves an activation across a BF16 rounding boundary now and then (measured 1.7e-5)
    assert err <= 1e-3
    # sub-range
    loss2, g2 = tr.loss_grad(100, 500)
    loss2_o, g2_o, _ = M.forward_backward(p, X[100:600], t[100:600])
    assert np.linalg.norm(g2 - g2_o) / np.linalg.norm(g2_o) <= 1e-3


def test_training_reduces_loss_and_predict_matches_oracle():
    X, t = data(20000)
    tr = T.MlpTrainer(X, t, seed=3)
    l0, _ = tr.loss_grad()
    losses = tr.train(epochs=20, batch=1024, lr=3e-3)
    l1, _ = tr.loss_grad()
    assert l1 < 0.2 * l0, (l0, l1, losses)
    p = tr.params()
    y = tr.predict(X[:500])
    _, _, y_o = M.forward_backward(p, X[:500], t[:500])
    assert np.max(np.abs(y - y_o)) <= 2e-2 * max(1.0, np.abs(y_o).max())


def small_channel(precision="f32", cs=0.0, omega=None):
    g = G.sphere_in_box(32, 16, 40, 3, 16, 8, 12, walls=True)
    p = G.params_lattice_units(g, "D3Q19", 0.05, 60.0, 6.0, 50, cs=cs)
    if omega is not None:
        p.omega = omega
    return g, p


def test_constant_closure_equals_bgk_at_that_rate():
    """w3 = 0, b3 = c: the network returns nu_t = out_scale * c everywhere, so the learned
    closure must reproduce plain BGK at tau = 3 (nu + nu_t) + 1/2 on fluid nodes (inlet/outlet
    use the base rate in both runs when cs = 0)."""
    g, p = small_channel()
    nu = (1.0 / p.omega - 0.5) / 3.0
    params = M.init_params(2)
    params[M.OW3:M.OB3] = 0.0
    params[M.OB3] = 0.5
    out_scale = 0.02
    nu_t = out_scale * 0.5
    a = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f32",
                                    arithmetic="fast")
    a.set_closure_mlp(params, np.ones(8), np.zeros(8), out_scale, 0.5001)
    # reference: every node at tau_t (fluid) -- run with omega_t but keep the boundary rate by
    # comparing fluid-dominated interior fields after one step from rest
    a.run(0, 1)
    pb = G.params_lattice_units(g, "D3Q19", 0.05, 60.0, 6.0, 50)
    pb.omega = 1.0 / (3.0 * (nu + nu_t) + 0.5)
    b = T.TLBMPartition.from_arrays(T.problem_from_params(pb), g.nd_type, precision="f32",
                                    arithmetic="fast")
    b.run(0, 1)
    fa, fb = a.populations(1), b.populations(1)
    fluid = np.repeat(g.nd_type == G.FLUID, 19)
    assert np.max(np.abs(fa[fluid] - fb[fluid])) <= 2e-6


def test_box_filter_matches_numpy():
    g, p = small_channel()
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f32",
                                       arithmetic="fast")
    part.run(0, 30)
    ux, uy, uz, rho = [a.reshape(g.nz, g.ny, g.nx).astype(np.float64) for a in part.macros()]
    F = part.filtered_fields(4)

    def box(a):
        nz, ny, nx = a.shape
        return a.reshape(nz // 4, 4, ny // 4, 4, nx // 4, 4).mean(axis=(1, 3, 5))

    want = {"rho": box(rho), "ux": box(ux), "uy": box(uy), "uz": box(uz), "uxux": box(ux * ux),
            "uyuy": box(uy * uy), "uzuz": box(uz * uz), "uxuy": box(ux * uy),
            "uxuz": box(ux * uz), "uyuz": box(uy * uz)}
    for k, v in want.items():
        assert np.allclose(F[k], v, rtol=1e-5, atol=1e-9), k


def test_inlet_profile_sets_inlet_velocity():
    g, p = small_channel()
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f32",
                                       arithmetic="fast")
    prof = 0.05 * (1.0 + 0.01 * CL.inlet_noise(g.nx, g.ny))
    part.set_inlet_profile(prof)
    part.run(0, 3)
    uz = part.macros()[2].reshape(g.nz, g.ny, g.nx)
    inlet = g.nd_type.reshape(g.nz, g.ny, g.nx)[0] == G.INLET
    assert np.allclose(uz[0][inlet], prof.reshape(g.ny, g.nx)[inlet], rtol=1e-6)
    with pytest.raises(T.TLBMError):
        ref = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f64",
                                          arithmetic="reference")
        ref.set_inlet_profile(prof)


def test_closure_pipeline_small():
    """A miniature run of the whole pipeline (fine 64x32x32 -> coarse 32x16x16): the network
    trains on the GPU, the learned closure runs fused in collide, and its errors against the
    filtered fine run are reported next to Smagorinsky's and plain BGK's (mechanics only; the
    comparison is made at the configured size below)."""
    out, cl = CL.study(cx=32, cy=16, cz=16, factor=2, u_in=0.05, re=200.0, coarse_steps=256,
                       snap_every=32, train_from=96, epochs=15)
    print(out)
    assert out["fine_finite"]
    # the fine run's collision is reported, with its departure from plain BGK
    assert out["fine_run"]["collision"] == "smagorinsky" and out["fine_run"]["deviation"]
    assert out["loss_final"] < out["loss_initial"]
    assert out["learned"]["finite"] and out["smagorinsky"]["finite"]


def test_learned_closure_against_smagorinsky_les():
    """The closure experiment at its configured size (coarse 128x64x64 LES at Re 3000 against a
    4x finer run, box-filtered), on the held-out final snapshot:
      * the learned closure beats the reference's Smagorinsky model at its configured cs = 0.1
        (the sum of mean-profile and log-spectrum errors);
      * its network is used and changes the flow: the calibration keeps a non-zero output scale,
        and the result differs from its Smagorinsky floor alone (a zeroed network would give the
        floor's numbers exactly);
      * measured against Smagorinsky calibrated on the same snapshot over the same coefficients
        (which is also the floor alone here), it stays within 3 % on each error: at this
        resolution the network adds nothing measurable over a calibrated Smagorinsky (measured
        on GB300: spectrum 0.0935 vs 0.0919, profile 0.0472 vs 0.0473)."""
    out, cal = CL.study()
    err = lambda e: e["profile_err"] + e["spectrum_log_err"]
    L, F = out["learned"], out["floor_only"]
    S, SC = out["smagorinsky"], out["smagorinsky_calibrated"]
    print({k: out[k] for k in ("smagorinsky", "smagorinsky_calibrated", "learned", "floor_only")})
    print(out["calibration"]["floor_cs"], out["calibration"]["multiplier"])
    assert all(e["finite"] for e in (L, F, S, SC))
    assert err(L) < 0.6 * err(S)
    assert out["calibration"]["multiplier"] > 0
    assert (L["profile_err"], L["spectrum_log_err"]) != (F["profile_err"], F["spectrum_log_err"])
    assert L["profile_err"] <= 1.03 * SC["profile_err"]
    assert L["spectrum_log_err"] <= 1.03 * SC["spectrum_log_err"]


# lattice weights by |e|^2 (include/D3Q{15,19,27}LatticeStructure.hpp), as the kernels use them
WEIGHTS = {15: {0: 2 / 9, 1: 1 / 9, 3: 1 / 72}, 19: {0: 1 / 3, 1: 1 / 18, 2: 1 / 36},
           27: {0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}}


@pytest.mark.parametrize("q", [19, 15, 27])
def test_fused_tensor_core_closure_matches_oracle(q):
    """One step of the fused collide kernel with a random network, from a non-equilibrium state
    on an all-fluid periodic box, against the closure computed in numpy: moments, Pi_neq,
    normalised features, the BF16-rounded network (mlp_oracle), tau = 3 (nu + s y) + 1/2 and the
    BGK relaxation.  The network runs on the tensor cores in the kernel (mma.sync, FP32
    accumulation in another order); a wrong network output would move the populations of
    most nodes by ~1e-4."""
    nx, ny, nz = 64, 8, 6
    g = G.Geometry(nx, ny, nz, np.zeros(nx * ny * nz, np.int32))
    p = G.params_lattice_units(g, "D3Q%d" % q, 0.05, 60.0, 6.0, 10)
    p.omega = 1.6
    n = g.num_nodes
    part = T.TLBMPartition.from_arrays(T.problem_from_params(p), g.nd_type, precision="f32",
                                       arithmetic="fast")
    rng = np.random.default_rng(12)
    part.load_restart(rng.uniform(-0.04, 0.04, n), rng.uniform(-0.04, 0.04, n),
                      rng.uniform(-0.04, 0.04, n), rng.uniform(0.99, 1.01, n))
    part.run(0, 1)
    f = part.populations(0).reshape(n, q).astype(np.float64)  # input of the next step
    # lattice vectors from the neighbour table (push target of an interior node)
    c = 1 + nx + nx * ny
    tgt = part.adjacency().reshape(n, q)[c]
    e = np.stack([tgt % nx - 1, (tgt // nx) % ny - 1, tgt // (nx * ny) - 1], axis=1)
    w = np.array([WEIGHTS[q][int(k)] for k in (e * e).sum(1)], np.float32)
    w = w.astype(np.float64)
    rho = f.sum(1)
    u = (f @ e) / rho[:, None]
    eu = u @ e.T
    feq = w[None, :] * rho[:, None] * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * (u * u).sum(1)[:, None])
    d = f - feq
    pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
    pi = np.stack([(d * (e[:, a] * e[:, b])[None, :]).sum(1) for a, b in pairs], axis=1)
    pi_norm = np.sqrt((pi[:, :3] ** 2).sum(1) + 2 * (pi[:, 3:] ** 2).sum(1))
    raw = np.concatenate([pi, (rho - 1)[:, None], pi_norm[:, None]], axis=1)
    shift = raw.mean(0).astype(np.float32)
    scale = (1.0 / raw.std(0)).astype(np.float32)
    x = ((raw.astype(np.float32) - shift) * scale).astype(np.float32)
    params = M.init_params(21)
    _, _, y = M.forward_backward(params, x, np.zeros(n))
    out_scale = 0.01
    nu = (1.0 / p.omega - 0.5) / 3.0
    tau_min = 0.5001  # below every tau here: the rate follows the network in every cell
    tau = np.maximum(3.0 * (nu + out_scale * y) + 0.5, tau_min)
    assert tau.min() > tau_min and np.ptp(tau) > 1e-3
    part.set_closure_mlp(params, scale, shift, out_scale, tau_min)
    part.run(1, 1)
    got = part.populations(1).reshape(n, q).astype(np.float64)

    def rate_error(tau_of_cell):
        # the relaxation rate each node applied (least squares over its q speeds) against 1/tau
        om = ((f - got) * d).sum(1) / (d * d).sum(1)
        return np.abs(om * tau_of_cell - 1.0)

    rel = rate_error(tau)
    # control: a network whose output weights differ by 25 % must be told apart
    wrong = params.copy()
    wrong[M.OW3:M.OB3] *= 1.25
    _, _, y_w = M.forward_backward(wrong, x, np.zeros(n))
    rel_w = rate_error(np.maximum(3.0 * (nu + out_scale * y_w) + 0.5, tau_min))
    print("fused closure step D3Q%d: rate error median %.2e, 99th pct %.2e; perturbed network "
          "median %.2e" % (q, np.median(rel), np.percentile(rel, 99), np.median(rel_w)))
    # the kernel's activation rounds the special-function unit's FP32 tanh (relative error below
    # 2^-10.9) to BF16, which differs from the oracle's BF16 of the exact tanh by one BF16 ulp
    # (2^-8 relative) only where the two straddle a rounding boundary; FP32 round-off of the
    # populations adds ~1e-7 to the rate (measured: median 3.5e-7, 99th percentile 4.5e-5)
    assert np.median(rel) <= 1e-5
    assert np.percentile(rel, 99) <= 1e-3
    assert np.median(rel_w) >= 10 * np.median(rel)
