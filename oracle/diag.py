"""The reference's interface-plane energies restated in numpy, in its order of
summation (avestrain F:641-749 for the plane sums, ResidualEnergy F:3920-3945
for the line), from Re xi of a state.

TEST INFRASTRUCTURE ONLY: the oracle of the diagnostics tests; the product
never imports it."""
import numpy as np


def plane_points(n, ppoint, normal):
    """avestrain's plane test (F:691, F:702) in its row-major loop order."""
    pts = []
    for k1 in range(n[0]):
        for k2 in range(n[1]):
            for k3 in range(n[2]):
                if (abs(normal[0] * (k1 - ppoint[0]) + normal[1] * (k2 - ppoint[1]) + normal[2] * (k3 - ppoint[2]))
                        <= 1.0 and k1 == ppoint[0]):
                    pts.append((k1, k2, k3))
    return pts


def compliance(S11, S12, S44):
    d = lambda i, j: 1 if i == j else 0
    d4 = lambda i, j, k, l: 1 if (i == j and j == k and k == l) else 0
    S = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    S[i, j, k, l] = ((S11 + 2 * S12) / 3.0 * d(i, j) * d(k, l)
                                     + S44 / 4.0 * (d(i, k) * d(j, l) + d(i, l) * d(j, k)) - S44 / 2.0 * d4(i, j, k, l)
                                     + (S11 - S12) * (d4(i, j, k, l) - d(i, j) * d(k, l) / 3.0))
    return S


def energies(re_xi, eps, p):
    """[energy_in, energy_in2, energy_in3, energy_in4 (one call), energy_Residual, total]
    of the state re_xi [ns, n1, n2, n3]; p: a native.DiagParams."""
    ns, n = re_xi.shape[0], re_xi.shape[1:]
    pp = list(p.ppoint)
    sig = np.array(list(p.sigma)).reshape(3, 3)
    S = compliance(p.S11, p.S12, p.S44)
    e3 = e4 = 0.0
    for (k1, k2, k3) in plane_points(n, pp, list(p.interface_n)):
        sp = np.zeros((3, 3))
        for u in range(3):
            for v in range(3):
                acc = 0.0
                for a in range(ns):
                    acc += re_xi[a, k1, k2, k3] * eps[a, u, v]
                sp[u, v] = acc
        for i in range(3):
            for j in range(3):
                e3 += -(sp[i, j] + 0.0) * sig[i, j]
                for k in range(3):
                    for l in range(3):
                        e4 += -S[i, j, k, l] * sig[k, l] * sig[i, j] * 0.5 * p.mu
    D00, D01, D10, D11 = list(p.D)
    nspm = p.ns_per_material or ns
    er = 0.0
    with np.errstate(invalid="ignore"):
        for j in range(n[1]):
            x0 = x1 = 0.0
            for a in range(ns):
                if a // nspm == 0:
                    x0 += re_xi[a, pp[0], j, pp[2]]
                if a // nspm == 1:
                    x1 += re_xi[a, pp[0], j, pp[2]]
            er = er + abs(-D11 * x1 * x1 + (D10 + D01) * x1 * x0 - D00 * x0 * x0)
    out = [0.0, 0.0, e3, e4, er]
    return np.array(out + [out[0] + out[1] + out[2] + out[3] + out[4]])
