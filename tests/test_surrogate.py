"""HLLD flux surrogate: the CPU oracle (oracle/mlp_oracle.c) pinned by finite
differences; on the GPU the encoding, harvested dissipation targets,
gradients and the tensor-core forward pass against the oracle, training,
and the deployed network in the flux stage against the FP64 solution."""

import numpy as np
import pytest

from ppkmhd_gb300 import workloads

G = "1.6666666666666667"
GAMMA = workloads.f32(G)


def _random_faces(rng, n):
    """Plausible normal-frame face states (rho, vn, vt1, vt2, p, Bt1, Bt2), a."""
    ql = np.empty((n, 7))
    ql[:, 0] = rng.uniform(0.1, 3.0, n)
    ql[:, 1:4] = rng.normal(0, 1, (n, 3))
    ql[:, 4] = rng.uniform(0.05, 3.0, n)
    ql[:, 5:7] = rng.normal(0, 0.7, (n, 2))
    jump = rng.uniform(0, 0.08, (n, 1)) * rng.normal(0, 1, (n, 7))
    qr = ql * (1 + jump)
    qr[:, 1:4] = ql[:, 1:4] + jump[:, 1:4]
    a = rng.normal(0, 0.7, n)
    return ql, qr, a


# ---------------------------------------------------------------- CPU

def test_oracle_gradient_matches_finite_differences(oracle):
    rng = np.random.default_rng(0)
    P = rng.normal(0, 0.2, oracle.MLP_NPARAM)
    X = rng.normal(0, 1, (24, oracle.MLP_NFEAT))
    X[:, 27:32] = 0
    T = rng.normal(0, 1, (24, 8))
    T[:, 7] = 0
    _, g = oracle.mlp_loss_grad(P, X, T)
    for i in rng.choice(oracle.MLP_NPARAM, 60, replace=False):
        h = 1e-6
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += h
        Pm[i] -= h
        fd = (oracle.mlp_loss_grad(Pp, X, T)[0] - oracle.mlp_loss_grad(Pm, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_oracle_encoding_is_dimensionless(oracle):
    rng = np.random.default_rng(1)
    ql, qr, a = _random_faces(rng, 20)
    for s in range(20):
        f, sc, J = oracle.mlp_encode(ql[s], qr[s], a[s])
        # rho -> k rho, p -> k p, B -> sqrt(k) B leaves velocities and features unchanged
        k = 3.7
        sl = ql[s] * np.array([k, 1, 1, 1, k, np.sqrt(k), np.sqrt(k)])
        sr = qr[s] * np.array([k, 1, 1, 1, k, np.sqrt(k), np.sqrt(k)])
        f2, sc2, J2 = oracle.mlp_encode(sl, sr, a[s] * np.sqrt(k))
        assert np.allclose(f, f2, rtol=1e-12, atol=1e-12)
        assert abs(J - J2) < 1e-12
        assert np.allclose(sc2[[0, 2, 3, 4]], k * sc[[0, 2, 3, 4]], rtol=1e-12)


def test_oracle_network_is_odd_in_each_transverse_direction(oracle):
    """Reflecting t1 (vt1, Bt1 -> -vt1, -Bt1) flips the mt1 and Bt1
    dissipation and leaves the others, for any weights; a face without
    transverse components gets exactly zero transverse dissipation."""
    rng = np.random.default_rng(8)
    P = rng.normal(0, 0.3, oracle.MLP_NPARAM)
    ql, qr, a = _random_faces(rng, 16)
    for s in range(16):
        f, _, _ = oracle.mlp_encode(ql[s], qr[s], a[s])
        m = np.array([1, 1, -1, 1, 1, -1, 1.0])
        g, _, _ = oracle.mlp_encode(ql[s] * m, qr[s] * m, a[s])
        y = oracle.mlp_forward(P, f[None])[0]
        z = oracle.mlp_forward(P, g[None])[0]
        assert np.allclose(z[[0, 1, 2, 4, 6]], y[[0, 1, 2, 4, 6]], rtol=1e-13, atol=1e-15)
        assert np.allclose(z[[3, 5]], -y[[3, 5]], rtol=1e-13, atol=1e-15)
        m2 = np.array([1, 1, 1, 0, 1, 1, 0.0])  # no t2 components at all
        h, _, _ = oracle.mlp_encode(ql[s] * m2, qr[s] * m2, a[s])
        w = oracle.mlp_forward(P, h[None])[0]
        assert w[4] == 0.0 and w[6] == 0.0


def test_oracle_central_flux_is_hlld_for_equal_states(oracle):
    """Equal states: HLLD returns the physical flux, so D = 0
    (RiemannSolvers_MHD.h:133-367 samples the left state)."""
    p = oracle.params_from_ini(workloads.ot_ini(2, 16, gamma0=G))
    rng = np.random.default_rng(2)
    ql, _, a = _random_faces(rng, 10)
    for s in range(10):
        q8 = np.array([ql[s, 0], ql[s, 4], ql[s, 1], ql[s, 2], ql[s, 3], a[s], ql[s, 5], ql[s, 6]])
        fh = oracle.riemann(p, q8, q8)
        fc = oracle.mlp_central_flux(ql[s], ql[s], a[s], GAMMA)
        fh7 = fh[[0, 1, 2, 3, 4, 6, 7]]
        assert np.allclose(fc, fh7, rtol=1e-12, atol=1e-12)


def test_committed_weights_file():
    from ppkmhd_gb300 import surrogate

    z = np.load(surrogate.DEFAULT_WEIGHTS)
    assert z["params"].shape == (7832,) and z["params"].dtype == np.float32
    assert np.isfinite(z["params"]).all()
    assert abs(float(z["gamma0"]) - GAMMA) < 1e-12


# ---------------------------------------------------------------- GPU

def _records_from_solver(mhdlib, n=48, stride=1):
    s = mhdlib.MHDSolver.from_ini(workloads.ot_ini(2, n, gamma0=G, precision=32))
    s.init_problem()
    s.run(20)
    return s, s.harvest(stride)


@pytest.mark.gpu
def test_harvest_records_against_oracle(mhdlib, oracle):
    s, rec = _records_from_solver(mhdlib, n=40, stride=3)
    nface = 41 * 41
    assert rec.shape == (2 * ((nface + 2) // 3), 24)
    p = oracle.params_from_ini(workloads.ot_ini(2, 40, gamma0=G))
    rng = np.random.default_rng(3)
    for q in rng.choice(rec.shape[0], 200, replace=False):
        r = rec[q].astype(np.float64)
        ql, qr, a = r[0:7], r[7:14], r[14]
        f, sc, J = oracle.mlp_encode(ql, qr, a)
        assert abs(J - r[15]) <= 1e-6 * max(J, 1e-3)
        # D = central flux - HLLD, both FP64 from the recorded states
        l8 = np.array([ql[0], ql[4], ql[1], ql[2], ql[3], a, ql[5], ql[6]])
        r8 = np.array([qr[0], qr[4], qr[1], qr[2], qr[3], a, qr[5], qr[6]])
        fh = oracle.riemann(p, l8, r8)[[0, 1, 2, 3, 4, 6, 7]]
        D = oracle.mlp_central_flux(ql, qr, a, GAMMA) - fh
        assert np.allclose(r[16:23], D, rtol=1e-5, atol=1e-7 * np.abs(fh).max()), (q, r[16:23], D)
        assert r[23] == np.float32(GAMMA)


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle(mhdlib, oracle):
    from ppkmhd_gb300.surrogate import FluxMLP

    _, rec = _records_from_solver(mhdlib)
    m = FluxMLP(seed=3)
    f, t = m.encode(rec[:3000])
    # the GPU encoding equals the oracle's
    for q in range(0, 3000, 97):
        r = rec[q].astype(np.float64)
        fo, sc, J = oracle.mlp_encode(r[0:7], r[7:14], r[14])
        assert np.allclose(f[q], fo, rtol=1e-5, atol=1e-6)
        assert np.allclose(t[q, :7], r[16:23] / sc, rtol=1e-5, atol=1e-6)
    P = m.params.astype(np.float64)
    g, loss = m.gradient(f, t, mode=mhdlib.MHD_MLP_CHECK)
    lo, go = oracle.mlp_loss_grad(P, f.astype(np.float64), t.astype(np.float64))
    assert abs(loss - lo) <= 1e-5 * lo
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
    # deployed numerics (BF16, hardware tanh): same direction
    g2, _ = m.gradient(f, t, mode=mhdlib.MHD_MLP_TRAIN)
    assert np.dot(g2, go) / (np.linalg.norm(g2) * np.linalg.norm(go)) > 0.99


@pytest.mark.gpu
def test_tensor_core_forward_matches_oracle(mhdlib, oracle):
    from ppkmhd_gb300.surrogate import FluxMLP

    rng = np.random.default_rng(4)
    m = FluxMLP(seed=5)
    P = m.params.copy()
    P[P != 0] += rng.normal(0, 0.05, (P != 0).sum()).astype(np.float32)
    P[32 * 64:33 * 64] = rng.normal(0, 0.3, 64)  # non-trivial b1
    m.params = P
    X = rng.normal(0, 1, (1000, 40)).astype(np.float32)
    X[:, 27:32] = 0
    y = m.forward(X).astype(np.float64)  # the tcgen05 batch forward (TMEM accumulators)
    yo = oracle.mlp_forward(m.params.astype(np.float64), X.astype(np.float64), rounding=True)
    yx = oracle.mlp_forward(m.params.astype(np.float64), X.astype(np.float64), rounding=False)
    err = np.sqrt(np.mean((y - yo) ** 2)) / np.sqrt(np.mean(yo ** 2))
    assert err < 1e-2, err
    # and the BF16 network is close to the exact one
    assert np.sqrt(np.mean((y - yx) ** 2)) / np.sqrt(np.mean(yx ** 2)) < 5e-2


@pytest.mark.gpu
def test_training_reduces_loss(mhdlib):
    from ppkmhd_gb300.surrogate import FluxMLP, smooth

    _, rec = _records_from_solver(mhdlib, n=96)
    rec = smooth(rec)
    m = FluxMLP(seed=7)
    f, t = m.encode(rec)
    _, l0 = m.gradient(f, t, mode=mhdlib.MHD_MLP_TRAIN)
    hist = m.train(rec, epochs=12, batch=2048, lr=3e-3, seed=2)
    _, l1 = m.gradient(f, t, mode=mhdlib.MHD_MLP_TRAIN)
    assert np.all(np.diff(hist) < 0) and l1 < 0.6 * l0, (l0, l1, hist)


def _turbulence_case(n):
    ini = workloads.ot_ini(3, n, gamma0=G, precision=32)
    U = workloads.turbulence_3d(n, seed=11)
    return ini, U


@pytest.mark.gpu
def test_surrogate_flux_stage_against_fp64_oracle(mhdlib, oracle):
    """Ablation on the turbulence state (64^3, 40 steps): FP32 with HLLD and
    FP32 with the network, both against the FP64 oracle; the network keeps
    the error within 1e-3 relative L1 while answering most faces."""
    from ppkmhd_gb300.surrogate import FluxMLP

    n, steps = 64, 40
    ini, U = _turbulence_case(n)
    o = oracle.OracleSolver(ini.replace("precision=32", "precision=64"), nthreads=16)
    o.set_state(U)
    o.run(steps)
    ref = oracle.interior(o.get_state())

    def run(mlp):
        s = mhdlib.MHDSolver.from_ini(ini)
        s.set_state(U.astype(np.float32))
        if mlp is not None:
            s.set_surrogate(mlp, tau=0.01)
        m0, _, _ = s.diagnostics()
        assert s.run(steps) == steps
        m1, _, dmax = s.diagnostics()
        err = np.abs(mhdlib.interior(s.get_state()).astype(np.float64) - ref).sum(axis=(1, 2, 3))
        err /= np.abs(ref).sum(axis=(1, 2, 3))
        used, total = s.surrogate_stats() if mlp is not None else (0, 1)
        return err, used / max(total, 1), m0, m1, dmax, s

    e_plain, _, _, _, _, _ = run(None)
    mlp = FluxMLP.load()
    e_net, frac, m0, m1, dmax, s = run(mlp)
    print(f"\nrel L1 vs FP64: HLLD {e_plain.max():.2e}, network {e_net.max():.2e}; "
          f"faces by the network {frac:.1%}")
    assert e_net.max() <= 1e-3, e_net
    assert frac > 0.5
    assert abs(m1[0] - m0[0]) <= 1e-5 * abs(m0[0])  # conservative: one flux per face
    assert dmax < 1e-3
    assert "k_flux_mlp" in [k for k, _ in s.profile_step()]


@pytest.mark.gpu
def test_surrogate_step_host_slabs_match_run(mhdlib):
    """The host-buffer step in slabs with the network in the flux stage (one
    more launch before the edge stage) gives the state of a run() step from
    the same float state, bitwise."""
    from ppkmhd_gb300.surrogate import FluxMLP

    ini, U = _turbulence_case(24)
    mlp = FluxMLP.load()
    a = mhdlib.MHDSolver.from_ini(ini)
    c = mhdlib.MHDSolver.from_ini(ini)
    for s in (a, c):
        s.set_state(U.astype(np.float32))
        s.set_surrogate(mlp, tau=0.01)
    c.set_host_slabs(3)
    V = c.get_state()
    out = np.zeros_like(V)
    for q in range(3):
        # a host state starts without low parts: compare with one run() step
        # from the same float state
        a.set_state(V)
        a.run(1)
        c.step_host(V, out)
        assert np.array_equal(mhdlib.interior(a.get_state()), mhdlib.interior(out)), q
        V, out = out, V


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 127, 128, 257, 1000, (1 << 20) + 77])
def test_tensor_core_forward_forms_bitwise(mhdlib, n):
    """The persistent two-pipeline forward and the one-tile-per-block forward
    give bitwise the same outputs, on ragged sizes and on more tiles than
    the persistent grid holds (each pipeline then loops over tiles)."""
    from ppkmhd_gb300.surrogate import FluxMLP

    rng = np.random.default_rng(n)
    m = FluxMLP(seed=7)
    P = m.params.copy()
    P[P != 0] += rng.normal(0, 0.05, (P != 0).sum()).astype(np.float32)
    m.params = P
    X = rng.normal(0, 1, (n, 40)).astype(np.float32)
    X[:, 27:32] = 0
    m.set_forward_form(mhdlib.MHD_MLP_FORWARD_TILES)
    y_tiles = m.forward(X)
    assert m.last_forward_ms() > 0
    m.set_forward_form(mhdlib.MHD_MLP_FORWARD_PERSISTENT)
    y_pers = m.forward(X)
    assert m.last_forward_ms() > 0
    assert np.isfinite(y_pers).all()
    assert np.array_equal(y_pers, y_tiles)


@pytest.mark.gpu
@pytest.mark.parametrize("form", [0, 1])
def test_tensor_core_wait_limit_reports_and_recovers(mhdlib, form):
    """A tensor-core completion wait that gives up is reported as an error
    (after the pending work drained), and the next call works again; in
    both kernel forms."""
    from ppkmhd_gb300.surrogate import FluxMLP

    m = FluxMLP(seed=3)
    m.set_forward_form(form)
    X = np.random.default_rng(1).normal(0, 1, (300, 40)).astype(np.float32)
    X[:, 27:32] = 0
    y0 = m.forward(X)
    m.set_wait_limit(0)
    with pytest.raises(mhdlib.MHDError) as e:
        m.forward(X)
    assert e.value.code == mhdlib.MHD_ERR_CUDA
    assert "wait" in str(e.value)
    m.set_wait_limit()
    assert np.array_equal(m.forward(X), y0)
