"""Independent vectorised numpy restatement of the FLUE path observables,
used only to cross-check the C oracle (two restatements written in different
styles must agree).  Fields are data[t,x,y,z,mu,a,b]; directions 1-based."""
import numpy as np

K5 = 1.0 / 180.0
K1 = 19.0 / 9.0 - 55.0 * K5
K2 = 1.0 / 36.0 - 16.0 * K5
K3 = 64.0 * K5 - 32.0 / 45.0
K4 = 1.0 / 15.0 - 6.0 * K5


def shift(f, off):
    """f(x + off) for a field indexed [t,x,y,z,...]"""
    return np.roll(f, shift=tuple(-int(o) for o in off), axis=(0, 1, 2, 3))


def dag(m):
    return np.conj(np.swapaxes(m, -1, -2))


def path_product(U, path):
    """Ordered product along path at every site (NOT transposed)."""
    shape = U.shape[:4]
    P = np.broadcast_to(np.eye(3, dtype=np.complex128), shape + (3, 3)).copy()
    pos = np.zeros(4, dtype=int)
    for st in path:
        mu = abs(st) - 1
        if st > 0:
            P = P @ shift(U[..., mu, :, :], pos)
            pos[mu] += 1
        else:
            pos[mu] -= 1
            P = P @ dag(shift(U[..., mu, :, :], pos))
    return P


def genericpath_all(U, path):
    return np.swapaxes(path_product(U, path), -1, -2)


def rect_leaves(mu, nu, a, b):
    """The four counter-clockwise a x b leaves at a site (a along mu)."""
    M = [mu] * a
    N = [nu] * b
    mM = [-mu] * a
    mN = [-nu] * b
    return [M + N + mM + mN, N + mM + mN + M, mM + mN + M + N, mN + M + N + mM]


def loop5_q(U, mu, nu):
    """Q (un-projected, un-transposed sum of leaves) of Loop5MuNuCoord."""
    q = 0
    for a, b, c in ((1, 1, K1), (2, 2, K2), (3, 3, K5), (1, 2, K3 / 2), (2, 1, K3 / 2), (1, 3, K4 / 2),
                    (3, 1, K4 / 2)):
        for p in rect_leaves(mu, nu, a, b):
            q = q + c * path_product(U, p)
    return q


def clover_q(U, mu, nu):
    q = 0
    for p in rect_leaves(mu, nu, 1, 1):
        q = q + path_product(U, p)
    return q


def ah_quarter(q):
    return 0.25 * 0.5 * (q - dag(q))


def loop5munucoord(U, mu, nu):
    return np.swapaxes(ah_quarter(loop5_q(U, mu, nu)), -1, -2)


def cloverloopmunucoord(U, mu, nu):
    return np.swapaxes(ah_quarter(clover_q(U, mu, nu)), -1, -2)


def magnetic(U):
    s = 0.0
    for mu, nu in ((3, 2), (2, 4), (4, 3)):
        f = loop5munucoord(U, mu, nu)
        s -= np.einsum("...ij,...ji->...", f, f).real.sum()
    return s / np.prod(U.shape[:4])


def plaquette(U, mustart, muend, nuend):
    s = 0.0
    n = 0
    for mu in range(mustart, muend + 1):
        for nu in range(mu + 1, nuend + 1):
            P = path_product(U, [mu, nu, -mu, -nu])
            s += np.trace(P, axis1=-2, axis2=-1).real.sum()
            n += np.prod(U.shape[:4])
    return s, n


def polyakov(U):
    nt = U.shape[0]
    P = U[0, ..., 0, :, :]
    for t in range(1, nt):
        P = P @ U[t, ..., 0, :, :]
    tr = np.trace(P, axis1=-2, axis2=-1)
    return tr.real.sum(), tr.imag.sum(), int(np.prod(U.shape[1:4]))


def wmunu(U, mu, nu, nmu, nnu):
    p = [mu] * nmu + [nu] * nnu + [-mu] * nmu + [-nu] * nnu
    P = path_product(U, p)
    return np.trace(P, axis1=-2, axis2=-1).real.mean()


def expm_su3(X):
    """exp of anti-Hermitian matrices via the eigen-decomposition of -iX."""
    w, v = np.linalg.eigh(-1j * X)
    return np.einsum("...ij,...j,...kj->...ik", v, np.exp(1j * w), np.conj(v))
