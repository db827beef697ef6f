"""Pair-form algebra of the contractions that run over symmetric pairs (ladder_sym.cu),
restated in numpy on the CPU: the pp ladder and Z[i][j][k][a] = sum_cd (kd|ac) tau[i][j][c][d].

tau+ / tau- are the ladder's packs of tau over its four symmetric partners; V+ / V- are
the packs of V[(k,a)][c,d] = (kd|ac) over c >= d / c > d.  Z is then
Zs = V+ tau+^T, Za = V- tau-^T with Z[i][j] = Zs + Za, Z[j][i] = Zs - Za (i > j), equal to
the plain contraction on tau with tau[i][j][c][d] = tau[j][i][d][c]."""
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
