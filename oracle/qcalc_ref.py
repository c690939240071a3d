"""CPU restatement of qcalc's calculations (TEST INFRASTRUCTURE; parity unpinned
by reference data: the reference ships no qcalc test output).

Only the tests load this file, as the checker of qsource_gb300's qgpu_calc_*
entry points.  Each function follows one calc_* module of the reference
(qusers/qsource, Q 5.06) frame by frame, in plain numpy:
  rms   calc_rms.f90 rms_calc      sqrt(sum((x - x0)**2) / n), no fit
  com   calc_com.f90 COM_calc      dot_product(x, mass) / total mass
  rmsf  calc_rmsf.f90 RMSF_calc    running mean / mean square per atom
  fit   calc_fit.f90 fit_calc      mass-weighted least-squares superposition
  geom  calc_geom.f90 dist_calc / angle_calc / torsion_calc (degrees)
  rdf   calc_rdf.f90 rdf_make_list + RDF_calc: the pair distance in real(4)
        (the FP64 difference rounded to single precision, minimum image in
        double rounded again, dot product and sqrt in single precision),
        bin int(dist/radius*Nbins + 1) in double
The reference ships no qcalc test data, so these restatements are the pin.
"""
import math

import numpy as np


def rms(frames, mask, x0):
    out = []
    m = np.asarray(mask)
    x0 = np.asarray(x0, dtype=np.float64).reshape(-1, 3)[m]
    for fr in np.asarray(frames, dtype=np.float64):
        x = fr.reshape(-1, 3)[m]
        out.append(math.sqrt(float(np.sum((x - x0) ** 2)) / len(m)))
    return np.array(out)


def rmsf(frames, mask):
    """calc_rmsf.f90 RMSF_calc (:56-80), frame by frame: x2 += x**2,
    x0 = x0*(1 - 1/n) + x/n, rmsf(atom) = sqrt(1/n*sum(x2) - sum(x0**2)),
    the printed value (1/N)*sum(rmsf) over the mask after each frame."""
    fr = np.asarray(frames, dtype=np.float64)
    nf = fr.shape[0]
    fr = fr.reshape(nf, -1, 3)
    m = np.asarray(mask)
    x0 = np.zeros((len(m), 3))
    x2 = np.zeros((len(m), 3))
    out = np.zeros(nf)
    for f in range(nf):
        n = float(f + 1)
        x = fr[f, m]
        x2 = x2 + x ** 2
        x0 = x0 * (1.0 - 1.0 / n) + x / n
        r = np.sqrt(1.0 / n * x2.sum(axis=1) - (x0 ** 2).sum(axis=1))
        out[f] = 1.0 / len(m) * r.sum()
    return out


def fit(frames, nsol, mask, mass, xref):
    """calc_fit.f90 fit_calc + LSQSTR, frame by frame: centre the solute on the
    mask's centre of mass, weight by sqrt(mass), U = sum over the mask of
    X XP^T, rotation R = B diag(1, 1, sign det U) A^T from the singular value
    decomposition U = A S B^T (the three largest eigenpairs of [[0, U],
    [U^T, 0]] in LSQSTR), X <- R X, x = X/sqrt(m) + xrcm.  Status 1 when
    |det U| < 1e-9, 2 when det U < 0 and the two smallest singular values are
    within 1e-5: the frame is then only moved to xrcm."""
    fr = np.asarray(frames, dtype=np.float64)
    nf = fr.shape[0]
    fr = fr.reshape(nf, -1, 3)
    m = np.asarray(mask)
    ms = np.asarray(mass, dtype=np.float64)
    x0 = np.asarray(xref, dtype=np.float64).reshape(-1, 3)
    sq = np.sqrt(ms[:nsol])[:, None]
    xrcm = (x0[m] * ms[m][:, None]).sum(axis=0) / ms[m].sum()
    xp = (x0[:nsol] - xrcm) * sq
    out = fr.copy()
    status = np.zeros(nf, dtype=np.int32)
    for f in range(nf):
        x = fr[f]
        xcm = (x[m] * ms[m][:, None]).sum(axis=0) / ms[m].sum()
        X = (x[:nsol] - xcm) * sq
        U = X[m].T @ xp[m]
        du = np.linalg.det(U)
        R = np.eye(3)
        if abs(du) < 1e-9:
            status[f] = 1
        else:
            a, sv, bt = np.linalg.svd(U)
            if du < 0 and abs(sv[1] - sv[2]) < 1e-5:
                status[f] = 2
            else:
                R = bt.T @ np.diag([1.0, 1.0, np.sign(du)]) @ a.T
        out[f, :nsol] = (X @ R.T) / sq + xrcm
    return out.reshape(nf, -1), status


def com(frames, mask, mass):
    m = np.asarray(mask)
    w = np.asarray(mass, dtype=np.float64)[m]
    out = []
    for fr in np.asarray(frames, dtype=np.float64):
        x = fr.reshape(-1, 3)[m]
        out.append([float(np.dot(x[:, c], w)) / float(np.sum(w)) for c in range(3)])
    return np.array(out)


def geom(frames, measurements):
    out = np.zeros((len(frames), len(measurements)))
    for f, fr in enumerate(np.asarray(frames, dtype=np.float64)):
        x = fr.reshape(-1, 3)
        for k, at in enumerate(measurements):
            if len(at) == 2:
                rji = x[at[0]] - x[at[1]]
                out[f, k] = math.sqrt(float(np.dot(rji, rji)))
            elif len(at) == 3:
                rji, rjk = x[at[0]] - x[at[1]], x[at[2]] - x[at[1]]
                scp = float(np.dot(rji, rjk)) / math.sqrt(float(np.dot(rji, rji)) * float(np.dot(rjk, rjk)))
                out[f, k] = math.degrees(math.acos(min(1.0, max(-1.0, scp))))
            else:
                rji, rjk, rkl = x[at[0]] - x[at[1]], x[at[2]] - x[at[1]], x[at[3]] - x[at[2]]
                rnj = np.cross(rji, rjk)
                rnk = -np.cross(rjk, rkl)
                scp = float(np.dot(rnj, rnk)) / math.sqrt(float(np.dot(rnj, rnj)) * float(np.dot(rnk, rnk)))
                phi = math.acos(min(1.0, max(-1.0, scp)))
                if float(np.dot(rjk, np.cross(rnj, rnk))) < 0:
                    phi = -phi
                out[f, k] = phi * 180.0 / math.pi
    return out


def rdf_counts(frames, mask1, mask2, radius, nbins, box=None):
    m1, m2 = np.asarray(mask1), np.asarray(mask2)
    counts = np.zeros(nbins, dtype=np.int64)
    for fr in np.asarray(frames, dtype=np.float64):
        x = fr.reshape(-1, 3)
        a, b = x[m1][:, None, :], x[m2][None, :, :]
        d = (a - b).astype(np.float32)                    # FP64 difference -> real(4)
        if box is not None:
            L = np.asarray(box, dtype=np.float64)
            dd = d.astype(np.float64)
            # delta - boxlength*nint(delta/boxlength), nint rounding halves away from zero
            n = np.sign(dd / L) * np.floor(np.abs(dd / L) + 0.5)
            d = (dd - L * n).astype(np.float32)
        r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
        dist = np.sqrt(r2.astype(np.float32))
        same = m1[:, None] == m2[None, :]
        sel = (~same) & (dist.astype(np.float64) < radius)
        bins = (dist[sel].astype(np.float64) / radius * nbins + 1.0).astype(np.int64) - 1
        bins = bins[(bins >= 0) & (bins < nbins)]
        counts += np.bincount(bins, minlength=nbins)[:nbins]
    return counts
