"""Pair-form algebra of the contractions that run over symmetric pairs (ladder_sym.cu),
restated in numpy on the CPU: Z[i][j][k][a] = sum_cd (kd|ac) tau[i][j][c][d],
X[k][l][i][j] = sum_cd (kc|ld) tau[i][j][c][d] and the hh ladder
S[i][j][a][b] = sum_kl W[k][l][i][j] tau[k][l][a][b].

tau+ / tau- are the ladder's packs of tau over its four symmetric partners; V+ / V- are
the packs of an integral row V[r][c,d] over c >= d / c > d.  Z (and X) is then
Zs = V+ tau+^T, Za = V- tau-^T with Z[i][j] = Zs + Za, Z[j][i] = Zs - Za (i > j), equal to
the plain contraction on tau with tau[i][j][c][d] = tau[j][i][d][c].  The hh ladder adds
W+ tau+ and W- tau- (W+- the (k,l) packs of W) to the halves S+- the pp ladder unpacks."""
import numpy as np
import pytest


def tri_pairs(n, strict):
    return [(p, q) for p in range(n) for q in range(p if strict else p + 1)]


def tau_packs(tau):
    o, v = tau.shape[0], tau.shape[2]
    tp = np.array([[(tau[i, j, c, d] + tau[j, i, d, c] + tau[i, j, d, c] + tau[j, i, c, d]) / 4
                    for (c, d) in tri_pairs(v, False)] for (i, j) in tri_pairs(o, False)])
    tm = np.array([[(tau[i, j, c, d] + tau[j, i, d, c] - tau[i, j, d, c] - tau[j, i, c, d]) / 4
                    for (c, d) in tri_pairs(v, True)] for (i, j) in tri_pairs(o, True)])
    return tp, tm


def v_packs(ovvv):
    """V+[(k,a)][tri(c,d)], V-[(k,a)][stri(c,d)] from ovvv[k][d][a][c] = (kd|ac)."""
    o, v = ovvv.shape[0], ovvv.shape[1]
    V = np.einsum("kdac->kacd", ovvv).reshape(o * v, v, v)  # V[(k,a)][c][d] = (kd|ac)
    vp = np.array([[V[r, c, d] + V[r, d, c] if c > d else V[r, c, c] for (c, d) in tri_pairs(v, False)]
                   for r in range(o * v)])
    vm = np.array([[V[r, c, d] - V[r, d, c] for (c, d) in tri_pairs(v, True)] for r in range(o * v)])
    return vp, vm


def z_unpack(o, v, zs, za):
    Z = np.zeros((o, o, o * v))
    for i in range(o):
        for j in range(o):
            i1, j1 = max(i, j), min(i, j)
            z = zs[i1 * (i1 + 1) // 2 + j1].copy()
            if i != j:
                za_row = za[i1 * (i1 - 1) // 2 + j1]
                z += za_row if i > j else -za_row
            Z[i, j] = z
    return Z.reshape(o, o, o, v)


@pytest.mark.parametrize("o,v", [(1, 3), (2, 1), (3, 5), (4, 7)])
def test_z_pair_form_equals_plain(o, v):
    rng = np.random.default_rng(31 + o * 10 + v)
    t = rng.standard_normal((o, o, v, v))
    tau = 0.5 * (t + t.transpose(1, 0, 3, 2))  # tau[i][j][c][d] = tau[j][i][d][c]
    ovvv = rng.standard_normal((o, v, v, v))
    plain = np.einsum("kdac,ijcd->ijka", ovvv, tau)
    tp, tm = tau_packs(tau)
    vp, vm = v_packs(ovvv)
    zs = tp @ vp.T
    za = tm @ vm.T if tm.size and vm.size else np.zeros((o * (o - 1) // 2, o * v))
    np.testing.assert_allclose(z_unpack(o, v, zs, za), plain, rtol=0, atol=1e-13)


def test_z_pair_form_symmetrises_tau():
    """On a tau without the partner symmetry the pair form gives the plain contraction on
    (tau[i][j][c][d] + tau[j][i][d][c]) / 2, as the pair-form ladder does."""
    o, v = 3, 4
    rng = np.random.default_rng(5)
    tau = rng.standard_normal((o, o, v, v))
    ovvv = rng.standard_normal((o, v, v, v))
    sym = 0.5 * (tau + tau.transpose(1, 0, 3, 2))
    tp, tm = tau_packs(tau)
    vp, vm = v_packs(ovvv)
    np.testing.assert_allclose(z_unpack(o, v, tp @ vp.T, tm @ vm.T), np.einsum("kdac,ijcd->ijka", ovvv, sym),
                               rtol=0, atol=1e-13)


def row_packs(V):
    """V+[r][tri(c,d)], V-[r][stri(c,d)] of V[r][c][d] (the kernels' row_pair_pack)."""
    n, v = V.shape[0], V.shape[1]
    vp = np.array([[V[r, c, d] + V[r, d, c] if c > d else V[r, c, c] for (c, d) in tri_pairs(v, False)]
                   for r in range(n)])
    vm = np.array([[V[r, c, d] - V[r, d, c] for (c, d) in tri_pairs(v, True)] for r in range(n)])
    return vp, vm.reshape(n, -1)


def x_unpack(o, xs, xa):
    """X[r][i][j] = Xs[r][tri(i,j)] + sgn(i-j) Xa[r][stri(i,j)] (pair index inner)."""
    X = np.zeros((o * o, o, o))
    for i in range(o):
        for j in range(o):
            i1, j1 = max(i, j), min(i, j)
            x = xs[:, i1 * (i1 + 1) // 2 + j1].copy()
            if i != j:
                a = xa[:, i1 * (i1 - 1) // 2 + j1]
                x += a if i > j else -a
            X[:, i, j] = x
    return X.reshape(o, o, o, o)


@pytest.mark.parametrize("o,v", [(1, 4), (3, 1), (3, 5), (4, 6)])
def test_x_pair_form_equals_plain(o, v):
    rng = np.random.default_rng(71 + o * 10 + v)
    t = rng.standard_normal((o, o, v, v))
    tau = 0.5 * (t + t.transpose(1, 0, 3, 2))
    ovov = rng.standard_normal((o, v, o, v))  # ovov[k][c][l][d] = (kc|ld)
    plain = np.einsum("kcld,ijcd->klij", ovov, tau)
    up, um = row_packs(np.einsum("kcld->klcd", ovov).reshape(o * o, v, v))
    tp, tm = tau_packs(tau)
    xs = up @ tp.T
    xa = um @ tm.T if tm.size and um.size else np.zeros((o * o, o * (o - 1) // 2))
    np.testing.assert_allclose(x_unpack(o, xs, xa), plain, rtol=0, atol=1e-13)


def ladder_unpack(o, v, sp, sm):
    """R[i][j][a][b] = S+[tri(i,j)][tri(a,b)] + sgn(i-j) sgn(a-b) S-[stri(i,j)][stri(a,b)]."""
    sg = lambda p, q: (p > q) - (p < q)
    R = np.zeros((o, o, v, v))
    for i in range(o):
        for j in range(o):
            i1, j1 = max(i, j), min(i, j)
            for a in range(v):
                for b in range(v):
                    a1, b1 = max(a, b), min(a, b)
                    x = sp[i1 * (i1 + 1) // 2 + j1, a1 * (a1 + 1) // 2 + b1]
                    s = sg(i, j) * sg(a, b)
                    if s:
                        x += s * sm[i1 * (i1 - 1) // 2 + j1, a1 * (a1 - 1) // 2 + b1]
                    R[i, j, a, b] = x
    return R


@pytest.mark.parametrize("o,v", [(1, 3), (2, 1), (3, 4), (4, 5)])
def test_hh_ladder_pair_form_equals_plain(o, v):
    rng = np.random.default_rng(97 + o * 10 + v)
    t = rng.standard_normal((o, o, v, v))
    tau = 0.5 * (t + t.transpose(1, 0, 3, 2))
    w = rng.standard_normal((o, o, o, o))
    W = 0.5 * (w + w.transpose(1, 0, 3, 2))  # W[k][l][i][j] = W[l][k][j][i]
    plain = np.einsum("klij,klab->ijab", W, tau)
    # W+-[pair(i,j)][pair(k,l)] for i >= j (i > j): the (k,l) packs of W[., ., i, j]
    rows_p = [(i, j) for (i, j) in tri_pairs(o, False)]
    rows_m = [(i, j) for (i, j) in tri_pairs(o, True)]
    wp = row_packs(np.array([W[:, :, i, j] for (i, j) in rows_p]))[0]
    wm = row_packs(np.array([W[:, :, i, j] for (i, j) in rows_m]))[1] if rows_m else np.zeros((0, 0))
    tp, tm = tau_packs(tau)
    sp = wp @ tp
    sm = wm @ tm if wm.size and tm.size else np.zeros((len(rows_m), v * (v - 1) // 2))
    np.testing.assert_allclose(ladder_unpack(o, v, sp, sm), plain, rtol=0, atol=1e-13)
