"""CPU restatement of the reference's spinor filter (spinors/filterSpinors/):
neighbour lists, the spin-orbit operator in both forms, the spinor
Hamiltonian and the Newton filter with complex coefficients.
TEST INFRASTRUCTURE ONLY.

Only tests/ and bench.py's CPU-baseline leg use this module, as the checker;
the product applies the spin-orbit operator on the GPU (csrc/sep_spinor.cu).

Pinned against the reference's own init_list, nonlocal_potential,
nonlocal_potential_kb, hamiltonian and filter, compiled from its sources by
oracle/Makefile.ref (tests/golden/spinor_vso.npz, made by
tests/golden/make_spinor_fixture.py).

Spinors are 2 ngrid complex values: the spin-up grid, then the spin-down
grid (filterSpinors/hamiltonian.c:38-44).  The neighbour lists are
structured arrays with the fields of the reference's nlc_st
(filterSpinors/fd.h:55-60), natom x nnlc, nl[a] entries used per atom.
"""
import numpy as np

PIE = 3.14159265358979323846
TWOPI = 6.28318530717958647692
EPSDX = 1.0e-20

NLC_DTYPE = np.dtype([("jxyz", "<i8"), ("y10", "<c16"), ("y11", "<c16"), ("y1_1", "<c16"),
                      ("Vs0G1", "<f8"), ("Vs0G_2", "<f8"), ("r", "<f8"), ("r2_1", "<f8"),
                      ("r2", "<f8"), ("Vr", "<f8")])


def neighbour_lists(vx, vy, vz, rxyz, vso, rnlcut2, nnlc):
    """Grid points within sqrt(rnlcut2) of each atom with r, r^2, Vso(r) and
    the l = 1 harmonics, filterSpinors/init.c:114-181 (x fastest)."""
    tmp1 = 0.5 * np.sqrt(3.0 / PIE)
    tmp2 = 0.5 * np.sqrt(3.0 / TWOPI)
    tmp49 = 1.0 / 0.49
    nx, ny, nz = len(vx), len(vy), len(vz)
    nat = len(rxyz)
    nlc = np.zeros((nat, nnlc), dtype=NLC_DTYPE)
    nl = np.zeros(nat, dtype=np.int64)
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    jxyz = (nx * (ny * zz + yy) + xx).ravel()
    for a in range(nat):
        dz = (np.asarray(vz)[zz] - rxyz[a][2]).ravel()
        dy = (np.asarray(vy)[yy] - rxyz[a][1]).ravel()
        dx = (np.asarray(vx)[xx] - rxyz[a][0]).ravel()
        dxe, dye, dze = dx + EPSDX, dy + EPSDX, dz + EPSDX
        dr2 = dx * dx + dy * dy + dz * dz
        sel = dr2 < rnlcut2
        n = int(sel.sum())
        if n > nnlc:
            raise ValueError("nnlc too small")
        dx, dy, dz, dxe, dye, dze, dr2 = (v[sel] for v in (dx, dy, dz, dxe, dye, dze, dr2))
        e = nlc[a, :n]
        e["jxyz"] = jxyz[sel]
        e["Vr"] = vso[a] * np.exp(-tmp49 * dr2)
        e["r"] = np.sqrt(dr2)
        d1 = 1.0 / np.sqrt(dx * dx + dy * dy + dze * dze)
        y10 = tmp1 * dze * d1 + 0j
        d1 = 1.0 / np.sqrt(dxe * dxe + dy * dy + dz * dz)
        y11r, y1_1r = -tmp2 * dxe * d1, tmp2 * dxe * d1
        d1 = 1.0 / np.sqrt(dx * dx + dye * dye + dz * dz)
        e["y10"] = y10
        e["y11"] = y11r + 1j * (-tmp2 * dye * d1)
        e["y1_1"] = y1_1r + 1j * (-tmp2 * dye * d1)
        far = dr2 > EPSDX
        e["r2_1"] = np.where(far, d1 * d1, 0.0)
        e["r2"] = np.where(far, dr2, 1.0 / EPSDX)
        nl[a] = n
    return nlc, nl


def vso_gauss(psi, nlc, nl, sigma, dv, ngrid):
    """|psinl> = Vso |psi> with a Gaussian of width sigma for delta(r - r'),
    filterSpinors/hamiltonian.c:81-190."""
    psi = np.asarray(psi, dtype=np.complex128)
    up, dn = psi[:ngrid], psi[ngrid:]
    out = np.zeros(2 * ngrid, dtype=np.complex128)
    tmp = 0.5 / np.sqrt(TWOPI * sigma * sigma) * dv
    sigma_1 = np.sqrt(0.5) / sigma
    s2 = np.sqrt(2.0)
    for a in range(len(nl)):
        e = nlc[a, :nl[a]]
        j = e["jxyz"]
        r, r2, vr = e["r"], e["r2"], e["Vr"]
        k = (0.5 * (vr[:, None] + vr[None, :]) * np.exp(-((r[:, None] - r[None, :]) * sigma_1) ** 2)
             / (0.5 * (r2[:, None] + r2[None, :])))
        s = {}
        for m in ("y11", "y10", "y1_1"):
            s[m, "up"] = k @ (np.conj(e[m]) * up[j])
            s[m, "dn"] = k @ (np.conj(e[m]) * dn[j])
        t11, t10, t1_1 = tmp * e["y11"], tmp * e["y10"], tmp * e["y1_1"]
        out[j] += (t11 * s["y11", "up"] - t1_1 * s["y1_1", "up"]
                   + s2 * (t10 * s["y11", "dn"] + t1_1 * s["y10", "dn"]))
        out[ngrid + j] += (-t11 * s["y11", "dn"] - t1_1 * s["y1_1", "dn"]
                           + s2 * (t10 * s["y1_1", "up"] + t11 * s["y10", "up"]))
    return out


def vso_kb(psi, nlc, nl, elkb, dv, ngrid):
    """|psinl> = Vso |psi> in the Kleinman-Bylander form,
    filterSpinors/hamiltonian.c:193-401 (with its term-by-term coefficients)."""
    psi = np.asarray(psi, dtype=np.complex128)
    up, dn = psi[:ngrid], psi[ngrid:]
    out = np.zeros(2 * ngrid, dtype=np.complex128)
    nat = len(nl)
    s6, s3 = np.sqrt(2.0) / 6.0, np.sqrt(2.0) / 3.0
    for a in range(nat):
        e = nlc[a, :nl[a]]
        j = e["jxyz"]
        g1, g2 = e["Vs0G1"], e["Vs0G_2"]
        y10, y11, y1_1 = e["y10"], e["y11"], e["y1_1"]
        p = {}
        for gname, g in (("G1", g1), ("G_2", g2)):
            for m, y in (("10", y10), ("11", y11), ("1_1", y1_1)):
                p[gname, m, "up"] = np.sum(g * (np.conj(y) * up[j]))
                p[gname, m, "dn"] = np.sum(g * (np.conj(y) * dn[j]))
        el1, el2 = elkb[a] * dv, elkb[a + nat] * dv
        for key in p:
            p[key] = p[key] * (el1 if key[0] == "G1" else el2)
        P = lambda g, m, s: p[g, m, s]
        out[j] += (1.0 / 6.0 * g2 * (P("G_2", "1_1", "up") * y1_1)
                   + 1.0 / 3.0 * g2 * (P("G_2", "10", "up") * y10)
                   + 0.5 * g2 * (P("G_2", "11", "up") * y11)
                   + s6 * g2 * (P("G_2", "10", "dn") * y1_1)
                   + s6 * g2 * (P("G_2", "11", "dn") * y10)
                   - 2.0 / 3.0 * g1 * (P("G1", "1_1", "up") * y1_1)
                   - 1.0 / 3.0 * g1 * (P("G1", "10", "up") * y10)
                   + s3 * g1 * (P("G1", "10", "dn") * y1_1)
                   + s3 * g1 * (P("G1", "11", "dn") * y10))
        out[ngrid + j] += (1.0 / 6.0 * g2 * (P("G_2", "11", "dn") * y11)
                           + 1.0 / 3.0 * g2 * (P("G_2", "10", "dn") * y10)
                           - 0.5 * g2 * (P("G_2", "1_1", "dn") * y1_1)
                           + s6 * g2 * (P("G_2", "1_1", "up") * y10)
                           + s6 * g2 * (P("G_2", "10", "up") * y11)
                           + s3 * g1 * (P("G1", "1_1", "up") * y10)
                           + s3 * g1 * (P("G1", "10", "up") * y10)
                           - 1.0 / 3.0 * g1 * (P("G1", "10", "dn") * y10)
                           - 2.0 / 3.0 * g1 * (P("G1", "11", "dn") * y11))
    return out


def kinetic(x, ksqr, dims):
    """T x = IFFT(ksqr FFT x) on one complex grid (x fastest); ksqr carries
    the 1/N of the unnormalised inverse, filterSpinors/hamiltonian.c:51-76."""
    nx, ny, nz = dims
    f = np.fft.fftn(np.asarray(x).reshape(nz, ny, nx)) * np.asarray(ksqr).reshape(nz, ny, nx)
    return (np.fft.ifftn(f) * (nx * ny * nz)).ravel()


def hamiltonian(psi, potl, ksqr, dims, nlc, nl, sigma, dv, flagkb=0, elkb=None):
    """H psi = T psi + V psi + Vso psi on a spinor (up grid, then down grid),
    filterSpinors/hamiltonian.c:8-46."""
    n = int(np.prod(dims))
    psi = np.asarray(psi, dtype=np.complex128)
    nlp = (vso_kb(psi, nlc, nl, elkb, dv, n) if flagkb else vso_gauss(psi, nlc, nl, sigma, dv, n))
    out = np.empty_like(psi)
    for s in (0, 1):
        part = psi[s * n:(s + 1) * n]
        out[s * n:(s + 1) * n] = kinetic(part, ksqr, dims) + (potl * part + nlp[s * n:(s + 1) * n])
    return out


def hnorm(psi, zm1, dE_1, vmin, *hargs, **hkw):
    """(H - z) psi in the filter's scaled form, filterSpinors/hnorm.c:5-17."""
    return dE_1 * hamiltonian(psi, *hargs, **hkw) - (2.0 + zm1 + vmin * dE_1) * psi


def newton_filter(start, an, zn, dE_1, vmin, *hargs, **hkw):
    """psims[e] = sum_j an[e, j] psi_j with psi_0 = start and
    psi_j = (H - z_{j-1}) psi_{j-1}; complex coefficients,
    filterSpinors/filter.c:48-80."""
    an = np.asarray(an)
    psi = np.asarray(start, dtype=np.complex128).copy()
    out = an[:, :1] * psi[None, :]
    for j in range(1, an.shape[1]):
        psi = hnorm(psi, zn[j - 1], dE_1, vmin, *hargs, **hkw)
        out += an[:, j:j + 1] * psi[None, :]
    return out


def _normalize(x, dv):
    """norm.c:27-44: x / sqrt(dv sum |x|^2)."""
    return x / np.sqrt(np.sum(x.real ** 2 + x.imag ** 2) * dv)


def energy(psi, dv, *hargs, **hkw):
    """Re <psi|H|psi> dv, filterSpinors/energy.c:5-20."""
    hp = hamiltonian(psi, *hargs, **hkw)
    return float(np.sum(psi.real * hp.real + psi.imag * hp.imag) * dv)


def energy_range(starts, dv, *hargs, tau=0.025, **hkw):
    """(Vmin, dE) of filterSpinors/energy.c:49-109: Emin by the damped
    iteration phi <- psi - tau H psi, Emax by power iteration, each to a
    relative change of 1e-6 or 500 steps; Emax * 1.2, Emin - 0.2 |Emin|.
    starts = the four normalised component grids that init_psi draws there
    (two spinors: Emin's, then Emax's)."""
    n = len(starts[0])
    phi = np.concatenate([starts[0], starts[1]]).astype(np.complex128)
    emin, old, i = 0.1, 0.0, 0
    while abs((emin - old) / emin) > 1.0e-6 and i < 500:
        psi = phi
        phi = _normalize(psi - tau * hamiltonian(psi, *hargs, **hkw), dv)
        old, emin = emin, energy(phi, dv, *hargs, **hkw)
        i += 1
    psi = np.concatenate([starts[2], starts[3]]).astype(np.complex128)
    emax, old, i = 0.1, 0.0, 0
    while abs((emax - old) / emax) > 1.0e-6 and i < 500:
        psi = _normalize(hamiltonian(psi, *hargs, **hkw), dv)
        old, emax = emax, energy(psi, dv, *hargs, **hkw)
        i += 1
    emax *= 1.2
    emin -= 0.2 * abs(emin)
    return emin, emax - emin


def pipeline(spinors, an, zn, dE_1, vmin, dv, *hargs, **hkw):
    """Filter every start spinor for all targets, normalise, orthogonalise
    (SVD, keep S_i / S_0 >= 1e-10), Rayleigh-Ritz and sigma:
    filterSpinors/main.c:92-131 with filter.c, norm.c:47-60, ortho.c:5-40,
    Hmat.c:5-75, energy.c:114-145.  Returns (eval, sigma)."""
    blocks = []
    for s in spinors:
        out = newton_filter(s, an, zn, dE_1, vmin, *hargs, **hkw)
        blocks.extend(_normalize(row, dv) for row in out)
    psi = np.array(blocks)                               # mstot x 2N
    u, sv, _ = np.linalg.svd(psi.T, full_matrices=False)
    keep = len(sv)
    for i in range(len(sv)):
        if sv[i] / sv[0] < 1.0e-10:
            keep = i
            break
    basis = np.array([_normalize(u[:, i], dv) for i in range(keep)])
    hb = np.array([hamiltonian(b, *hargs, **hkw) for b in basis])
    hm = (np.conj(basis) @ hb.T) * dv                    # <b_i|H|b_j>
    ev, vec = np.linalg.eigh(0.5 * (hm + np.conj(hm.T)))
    rot = vec.T @ basis
    rot = np.array([_normalize(r, dv) for r in rot])
    sig = []
    for r in rot:
        h1 = hamiltonian(r, *hargs, **hkw)
        h2 = hamiltonian(h1, *hargs, **hkw)
        e1 = np.sum(r.real * h1.real + r.imag * h1.imag) * dv
        e2 = np.sum(r.real * h2.real + r.imag * h2.imag) * dv
        sig.append(np.sqrt(abs(e2 - e1 * e1)))
    return ev, np.array(sig)
