"""Known-answer tests pinning the CPU oracle (the reference ships no tests or golden vectors)."""
import numpy as np
import pytest

from difftactile_gb300 import scene as S
from oracle import oracle as O


@pytest.mark.parametrize("dtype,tol", [(np.float32, 2e-6), (np.float64, 1e-13)])
def test_svd_convention_and_accuracy(dtype, tol):
    rng = np.random.default_rng(0)
    A = np.eye(3) + 0.3 * rng.standard_normal((4000, 3, 3))
    A[:4] = np.eye(3)
    A[4] = np.diag([1.0, 1.0, -1.0])
    A[5] = np.diag([2.0, 2.0, 1.0])
    A[6] = 0.0
    A[7] = np.diag([1.0, 0.5, 0.0])
    U, s, V = O.svd3(A, dtype)
    rec = np.einsum("nij,nj,nkj->nik", U, s, V)
    assert np.abs(rec - A).max() < 5 * tol * 10
    assert np.abs(np.einsum("nji,njk->nik", U, U) - np.eye(3)).max() < tol * 10
    assert np.abs(np.einsum("nji,njk->nik", V, V) - np.eye(3)).max() < tol * 10
    assert np.abs(np.linalg.det(U) - 1).max() < tol * 10  # det U = det V = +1 (ti.svd convention)
    assert np.abs(np.linalg.det(V) - 1).max() < tol * 10
    assert (s[:, :2] >= 0).all()
    assert np.all(np.abs(s[:, 0]) >= np.abs(s[:, 1]) - tol) and np.all(np.abs(s[:, 1]) >= np.abs(s[:, 2]) - tol)
    sv = np.linalg.svd(A, compute_uv=False)
    assert np.abs(np.abs(s) - sv).max() < tol * 10
    neg = np.linalg.det(A) < -1e-3
    assert (s[neg, 2] < 0).all()  # inverted elements keep the sign in the last singular value


def _svd_loss(A, W, sb, Rb):
    """sum_i <W_i, u_i v_i^T> + <sb, s> + <Rb, U V^T>: unchanged when the SVD flips the signs of a
    pair of matching columns, so central differences through svd3 are well defined."""
    U, s, V = O.svd3(A, np.float64)
    L = np.einsum("nkab,nak,nbk->n", W, U, V) + (sb * s).sum(1) + np.einsum("nab,nak,nbk->n", Rb, U, V)
    return L, U, s, V


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("det_sign", [1.0, -1.0])
def test_svd_adjoint_matches_finite_differences(mode, det_sign):
    """The SVD adjoint (svd_grad, mpm_elastic.py:145-173) on random F away from degeneracy (singular
    values at least 0.2 apart in magnitude), both the reference's form (mode 1, the R = U V^T adjoint
    folded into the U and V adjoints) and the divided form (mode 0), for det F > 0 and for inverted F
    (negative last singular value)."""
    rng = np.random.default_rng(3 + mode)
    n = 200
    Q1 = np.linalg.qr(rng.standard_normal((n, 3, 3)))[0]
    Q2 = np.linalg.qr(rng.standard_normal((n, 3, 3)))[0]
    sig = np.sort(rng.uniform(0.3, 2.0, (n, 3)), 1)[:, ::-1] + np.array([0.4, 0.2, 0.0])
    sig[:, 2] *= det_sign * np.sign(np.linalg.det(Q1) * np.linalg.det(Q2))
    A = np.einsum("nij,nj,nkj->nik", Q1, sig, Q2)
    W = rng.standard_normal((n, 3, 3, 3))     # W[:, k] weighs u_k v_k^T
    sb = rng.standard_normal((n, 3))
    Rb = rng.standard_normal((n, 3, 3))
    _, U, s, V = _svd_loss(A, W, sb, Rb)
    assert np.all(np.sign(np.linalg.det(A)) == det_sign)
    Ub = np.einsum("nkab,nbk->nak", W, V)      # d/du_k of <W_k, u_k v_k^T> = W_k v_k
    Vb = np.einsum("nkab,nak->nbk", W, U)      # d/dv_k = W_k^T u_k
    Fb = O.svd_grad(U, s, V, Ub, sb, Vb, Rb, mode)
    D = rng.standard_normal((n, 3, 3))
    eps = 1e-6
    fd = (_svd_loss(A + eps * D, W, sb, Rb)[0] - _svd_loss(A - eps * D, W, sb, Rb)[0]) / (2 * eps)
    pred = (Fb * D).sum((1, 2))
    assert np.abs(pred - fd).max() < 1e-6 * np.abs(fd).max()


def _cube(n=32, v=(0.0, 0.0, 0.0), gravity=(0, 0, 0), eps=1e-20, model=S.MODEL_COROTATED):
    x = S.cube_particles([0.5, 0.55, 0.45], 0.25, 1.0 / n, 8, 0)
    return S.EnvSpec(x=x, v=np.asarray(v, np.float32), materials=[S.Material(5e3, 0.3, 50.0, model)],
                     n_grid=(n, n, n), dx=1.0 / n, gravity=gravity, eps=eps, rho=1000.0)


@pytest.mark.parametrize("model", [S.MODEL_COROTATED, S.MODEL_VON_MISES, S.MODEL_NEOHOOKEAN])
def test_rest_state_stays_at_rest(model):
    env = _cube(eps=1e-5, model=model)
    o = O.Oracle(env, 1e-4)
    st = o.initial_state()
    st1, d = o.substep(st)
    assert d["err"] == 0
    for k in ("x", "F"):
        assert np.array_equal(st1[k], st[k])
    assert np.abs(st1["v"]).max() == 0 and np.abs(st1["C"]).max() == 0


@pytest.mark.parametrize("dtype,tol", [(np.float32, 3e-6), (np.float64, 1e-12)])
def test_rigid_translation(dtype, tol):
    v0 = np.array([0.3, -0.2, 0.1])
    o = O.Oracle(_cube(v=v0), 1e-4, dtype)
    st = o.initial_state()
    st1, d = o.substep(st)
    v0 = st["v"][0]
    assert np.abs(st1["v"] - v0).max() < tol * np.abs(v0).max() * 2
    assert np.abs(st1["C"]).max() < tol * 100
    assert np.abs(st1["x"] - (st["x"] + 1e-4 * st1["v"])).max() < tol
    # P2G conserves mass and momentum; partition of unity of the B-spline weights
    env = o.env
    assert abs(d["grid_m"].sum() / (env.p_mass * env.n_particles) - 1) < tol
    assert np.abs(d["grid_v_in"].reshape(-1, 3).sum(0) - env.p_mass * st["v"].sum(0)).max() < tol * env.p_mass * len(st["v"])


def test_free_fall():
    o = O.Oracle(_cube(v=(0.1, 0.0, 0.0), gravity=(0.0, -9.8, 0.0)), 1e-4, np.float64)
    st = o.initial_state()
    st1, _ = o.substep(st)
    assert np.abs(st1["v"] - (st["v"][0] + np.array([0.0, -9.8e-4, 0.0]))).max() < 1e-12
    assert np.abs(st1["x"] - st["x"] - 1e-4 * st1["v"]).max() < 1e-15


def test_momentum_conserved_without_external_forces():
    """Random velocities and deformation, no gravity, far from walls: total momentum is unchanged."""
    env = _cube()
    rng = np.random.default_rng(4)
    env = env.replace(v=0.2 * rng.standard_normal(env.x.shape).astype(np.float32))
    o = O.Oracle(env, 1e-4, np.float64)
    st = o.initial_state()
    st["F"] = st["F"] + 0.01 * rng.standard_normal(st["F"].shape)
    p0 = st["v"].sum(0)
    for _ in range(3):
        st, _ = o.substep(st)
    assert np.abs(st["v"].sum(0) - p0).max() < 1e-9 * np.abs(p0).max() * 1e3


def _single_tet_env(scale):
    verts = np.array([[0.5, 0.5, 0.5], [0.6, 0.5, 0.5], [0.5, 0.6, 0.5], [0.5, 0.5, 0.6]], np.float32)
    sp = S.SensorSpec(verts=verts, tets=np.array([[1, 2, 3, 0]], np.int32), tris=np.array([[1, 2, 3]], np.int32),
                      layer=np.ones(4, np.int32), mass=0.01, E=1e4, nu=0.3)
    env = S.EnvSpec(x=np.zeros((0, 3), np.float32), materials=[S.Material(1e3, 0.3)], n_grid=(8, 8, 8), dx=1 / 8,
                    sensors=[sp])
    o = O.Oracle(env, 1e-4, np.float64)
    st = o.initial_state()
    c = verts.mean(0)
    st["pos"] = [c + scale * (verts - c)]
    return o, st, sp


def test_fem_rest_tet_has_no_force():
    o, st, _ = _single_tet_env(1.0)
    _, d = o.substep(st)
    o2, st2, _ = _single_tet_env(1.1)
    _, d2 = o2.substep(st2)
    # stable-Neo-Hookean-like P at F = I: mu (1 - 1/4) I + lam (1 - alpha) I = 0 with alpha = 1 + 0.75 mu/lam;
    # what remains comes from the float32 rest-shape inverse
    assert np.abs(d["vel_mid"][0]).max() < 1e-5 * np.abs(d2["vel_mid"][0]).max()


def test_fem_uniform_dilation_matches_analytic_stress():
    s = 1.1
    o, st, sp = _single_tet_env(s)
    _, d = o.substep(st)
    mu, lam = sp.lame()
    alpha = 1 + 0.75 * mu / lam
    P = mu * (1 - 1 / (3 * s * s + 1)) * s + lam * (s ** 3 - alpha) * s * s  # P = p I
    verts = sp.verts.astype(np.float64)
    t = sp.tets[0]
    D = np.stack([st["pos"][0][t[k]] - st["pos"][0][t[3]] for k in range(3)], 1)
    Dm = np.stack([verts[t[k]] - verts[t[3]] for k in range(3)], 1)
    B = np.linalg.inv(Dm)
    H = -abs(np.linalg.det(D)) / 6 * P * B.T
    dv = np.zeros((4, 3))
    for k in range(3):
        dv[t[k]] += 1e-4 * H[:, k] / sp.mass
        dv[t[3]] -= 1e-4 * H[:, k] / sp.mass
    assert np.abs(d["vel_mid"][0] - dv).max() < 2e-6 * np.abs(dv).max()
    assert np.abs(dv.sum(0)).max() < 1e-12  # internal forces sum to zero


def _contact_env(v_block):
    n = 32
    dx = 1.0 / n
    lo = np.array([12, 4, 12]) * dx
    hi = np.array([20, 10, 20]) * dx
    x = S.box_particles(lo, hi, dx, 8, 0)
    pad = S.hex_pad_sensor([0.5, hi[1] + 0.5 * dx, 0.5], nx=10, nz=10, ny=2, h=dx)
    env = S.EnvSpec(x=x, v=np.asarray(v_block, np.float32), materials=[S.Material(5e3, 0.3)], n_grid=(n, n, n),
                    dx=dx, rho=1000.0, gravity=(0, 0, 0), eps=1e-20, sensors=[pad], kn=1e4, kd=100.0, kt=100.0,
                    mu_t=0.5)
    ys = float(pad.verts[pad.layer == pad.layer.max(), 1].mean())  # float32 surface height
    return env, pad, ys


@pytest.mark.parametrize("vt", [0.3, 1e-3])
def test_contact_force_known_answer(vt):
    """Flat pad at rest over a block sliding along x at rest state (no stress): every contacting node
    gets f_n = kn * depth * (-y) and a friction force opposite to its sliding, capped by mu |f_n|
    (grasp_plastic.py:205-216); contact forces on nodes and sensor vertices cancel."""
    env, pad, ys = _contact_env([vt, 0.0, 0.0])
    o = O.Oracle(env, 1e-4, np.float64)
    st = o.initial_state()
    _, d = o.substep(st)
    gf = d["grid_f"] / 1e-4
    hit = np.argwhere(np.abs(gf).sum(-1) > 0)
    assert len(hit) > 10
    for i, j, k in hit:
        yp = (j + 0.5) / 32
        depth = yp - ys
        assert depth > 0
        fn = 1e4 * depth
        ft = min(100.0 * float(np.float32(vt)), 0.5 * fn)
        np.testing.assert_allclose(gf[i, j, k], [-ft, -fn, 0.0], rtol=1e-6, atol=1e-9 * fn)
    np.testing.assert_allclose(gf.reshape(-1, 3).sum(0), -d["ext"][0].sum(0), rtol=1e-12, atol=1e-12)


def test_argmin_matches_brute_force():
    pad = S.hex_pad_sensor([0.5, 0.5, 0.5], nx=8, nz=8, ny=2, h=1 / 32)
    rng = np.random.default_rng(0)
    pos = pad.verts + 1e-3 * rng.standard_normal(pad.verts.shape).astype(np.float32)
    q = (rng.random((2000, 3)) * 0.5 + 0.25).astype(np.float32)
    got = O.find_closest(pad, pos, q)
    third = np.float32(1.0 / 3.0)
    t = pad.tris
    cent = third * ((pos[t[:, 0]] + pos[t[:, 1]]) + pos[t[:, 2]])
    d = cent[None, :, :] - q[:, None, :]
    dist = np.sqrt(((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]) + np.float32(1e-10))
    assert dist.dtype == np.float32
    np.testing.assert_array_equal(got, np.argmin(dist, 1))  # first minimum wins, like strict '<'


def test_dome_mesh_matches_reference_counts():
    """fem_sensor.py:293-322 with scipy's Delaunay: 1910 vertices, 8198 tets, 1543 surface triangles."""
    nodes, tets, tris, layer = S.dome_mesh()
    assert (len(nodes), len(tets), len(tris)) == (1910, 8198, 1543)
    assert (np.bincount(layer) == np.array([200, 355, 555, 800])).all()


def test_linear_corotated_tet_force_known_answer():
    """One tet of the linear corotated elastomer: the velocity change of its vertices is
    dt / m times -V0 P B^T (and minus their sum on the fourth vertex), P = 2 mu (F - R) + lam tr(R^T F - I) R
    with R the polar rotation of F = D B (scipy.linalg.polar), V0 the rest volume."""
    import scipy.linalg
    from difftactile_gb300 import scene as S_
    rest = np.array([[0.0, 0.0, 0.0], [0.02, 0.0, 0.0], [0.0, 0.02, 0.0], [0.0, 0.0, 0.02]], np.float32) + 0.4
    sp = S_.SensorSpec(verts=rest, tets=np.array([[1, 2, 3, 0]], np.int32), tris=np.zeros((0, 3), np.int32),
                       layer=np.ones(4, np.int32), mass=1e-3, E=1.5e5, nu=0.45, model=S_.FEM_LINEAR_COROTATED)
    env = S_.EnvSpec(x=np.zeros((0, 3), np.float32), materials=[S_.Material(5e3, 0.3)], n_grid=(16,) * 3,
                     dx=1 / 16, sensors=[sp], gravity=(0.0, 0.0, 0.0))
    rng = np.random.default_rng(2)
    pos = rest.astype(np.float64) + 0.002 * rng.standard_normal(rest.shape)
    o = O.Oracle(env, 1e-4, np.float64)
    st = o.initial_state()
    st["pos"] = [pos]
    _, d = o.substep(st)
    B = sp.rest_inverse()[0].astype(np.float64)
    t = sp.tets[0]
    D = np.stack([pos[t[k]] - pos[t[3]] for k in range(3)], 1)
    F = D @ B
    R, _ = scipy.linalg.polar(F)
    mu, lam = sp.lame()
    P = 2 * mu * (F - R) + lam * (np.trace(R.T @ F) - 3) * R
    H = -(1.0 / (6 * abs(np.linalg.det(B)))) * P @ B.T
    dv = np.zeros((4, 3))
    for k in range(3):
        dv[t[k]] += 1e-4 * H[:, k] / 1e-3
        dv[t[3]] -= 1e-4 * H[:, k] / 1e-3
    assert np.abs(dv).max() > 1e-3
    assert np.allclose(d["vel_mid"][0], dv, rtol=1e-9, atol=1e-12 * np.abs(dv).max())
