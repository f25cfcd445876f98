"""CPU restatement of the reference's bulk band-structure path
(pseudopotFitting/): TEST INFRASTRUCTURE ONLY.

Only tests/ and bench.py's CPU leg use this module, as the checker; the
product computes band structures on the GPU (csrc/sep_bulk.cu) and never
imports it.

Pinned against the reference's published runs (pseudopotFitting/TESTS,
tests/golden/bulk_fit.json): the zincblende CdSe band structure at its input
parameters and the wurtzite CdSe one at the fitted parameters printed in
output.dat, within the 5 printed decimals (eV).

Each function names the reference lines it restates.  The eigenvalues come
from numpy's LAPACK (eigvalsh) in place of MKL's zheev (diag.c:12-48).
"""
import numpy as np

AUTOEV = 27.2114          # fit.h AUTOEV
TWOPI = 6.28318530717958647692


def recip_vectors(cell):
    """b_i = 2 pi (a_j x a_k) / (a_0 . (a_1 x a_2)), init.c:21-45."""
    a = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    vol = a[0] @ np.cross(a[1], a[2])
    pre = TWOPI / vol
    return np.array([np.cross(a[1], a[2]) * pre, np.cross(a[2], a[0]) * pre,
                     np.cross(a[0], a[1]) * pre])


def basis(cell, max_ke):
    """Plane waves G = i b0 + j b1 + k b2 with G^2 / 2 < max_ke, states.c:10-61
    (ordered by |G|; the order within a shell does not change the spectrum)."""
    b = recip_vectors(cell)
    gmin = min(np.sqrt(v @ v) for v in b)
    n = int(np.sqrt(max_ke / (gmin * gmin))) + 1
    r = np.arange(-n, n + 1, dtype=np.float64)
    i, j, k = np.meshgrid(r, r, r, indexing="ij")
    g = (i.reshape(-1, 1) * b[0] + j.reshape(-1, 1) * b[1]) + k.reshape(-1, 1) * b[2]
    mag = np.sqrt(np.einsum("ij,ij->i", g, g))
    keep = 0.5 * mag * mag < max_ke
    g, mag = g[keep], mag[keep]
    return g[np.argsort(mag, kind="stable")]


def form_factor(q, a):
    """v(q) = a0 (q^2 - a1) / (a2 exp(a3 q^2) + 1), hamiltonian.c:91-94."""
    return a[0] * (q * q - a[1]) / (a[2] * np.exp(a[3] * q * q) + 1.0)


def potential_matrix(g, tau, atom_params):
    """V_jl = sum_a v_a(|G_j - G_l|) exp(-i (G_j - G_l) . tau_a) / natom,
    hamiltonian.c:55-83."""
    d = g[:, None, :] - g[None, :, :]
    q = np.sqrt(np.einsum("jlx,jlx->jl", d, d))
    na = len(tau)
    v = np.zeros(q.shape, dtype=np.complex128)
    for a in range(na):
        ph = np.einsum("jlx,x->jl", d, tau[a])
        v += form_factor(q, atom_params[a]) * (np.cos(ph) - 1j * np.sin(ph)) / na
    return v


def bands(cell, tau, atom_params, kpts, max_ke, nev, ke_scale=1.0, g=None):
    """Lowest nev eigenvalues (eV) of V + diag(ke_scale |k + G|^2 / 2) per
    k-point, fit.c:71-97 + hamiltonian.c:11-52 + diag.c:12-48."""
    if g is None:
        g = basis(cell, max_ke)
    v = potential_matrix(g, np.asarray(tau, dtype=np.float64), np.asarray(atom_params))
    out = np.zeros((len(kpts), nev))
    for ik, k in enumerate(np.asarray(kpts, dtype=np.float64)):
        kg = g + k
        h = v + np.diag(ke_scale * 0.5 * np.einsum("jx,jx->j", kg, kg))
        out[ik] = np.linalg.eigvalsh(h)[:nev] * AUTOEV
    return out


def band_weights(ne):
    """Per-band weights of fit.c:106-112 (band-edge bands weigh most)."""
    w = np.zeros(ne)
    for j in range(ne // 2):
        val = 0.06125 if j < ne // 8 else (2.0 if j < ne // 4 else 4.0)
        w[j] = w[ne - j - 1] = val
    return w


def weighted_mse(b, exp):
    """fit.c:125-145: targets with |E| <= 1e-10 are skipped."""
    b, exp = np.asarray(b), np.asarray(exp)
    w = np.broadcast_to(band_weights(b.shape[1]), b.shape)
    use = np.abs(exp) > 1e-10
    return float(np.sum(w[use] * (b[use] - exp[use]) ** 2) / np.count_nonzero(use))
