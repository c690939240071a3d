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
  com_ke calc_com_ke.f90 COM_KE_calc: translational and rotational kinetic
        energy of a mask's centre of mass from consecutive frames
  nb    calc_nb.f90 nb_make_list + nb_calc_lists: the pair list between two
        masks with its LJ and charge products, and per frame the summed
        LJ and Coulomb energies, in plain Python loops
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


def com_ke(frames, mask, mass, frame_length):
    """calc_com_ke.f90 COM_KE_calc (:156-298), frame by frame; the first
    frame is its own predecessor.  Per frame, with the mask's masses m and
    total M (COM_KE_put_mass :301-322):
      c, p = mass-weighted centres of this and the previous frame;
      rel = x - c, rel' = x' - p, v = (rel - rel')/dt;
      inertia tensor of rel (Ixx = sum m (y^2 + z^2), Ixy = -sum y x m, ...);
      its eigenpairs (I_j, e_j) (EIGEN, :227-233);
      rad_j = rel - (e_j . rel) e_j, L_j = sum (rad_j x v) m;
      rotational sum_j |L_j|^2/(2 I_j) * 2390, translational
      0.5 M |p - c|^2 / dt^2 * 2390 (the integer conversion factor, :33).
    Returns [nframes, 2] (translational, rotational)."""
    conv = 2390
    fr = np.asarray(frames, dtype=np.float64)
    nf = fr.shape[0]
    fr = fr.reshape(nf, -1, 3)
    mk = np.asarray(mask)
    m = np.asarray(mass, dtype=np.float64)[mk]
    M = 0.0
    for w in m:
        M += float(w)
    out = []
    prev = fr[0][mk]
    for f in range(nf):
        x = fr[f][mk]
        c = np.array([float(np.dot(x[:, r], m)) / M for r in range(3)])
        p = np.array([float(np.dot(prev[:, r], m)) / M for r in range(3)])
        rel, relp = x - c, prev - p
        Ixx = float(np.dot(rel[:, 1] ** 2 + rel[:, 2] ** 2, m))
        Iyy = float(np.dot(rel[:, 0] ** 2 + rel[:, 2] ** 2, m))
        Izz = float(np.dot(rel[:, 1] ** 2 + rel[:, 0] ** 2, m))
        Ixy = -float(np.sum(rel[:, 1] * rel[:, 0] * m))
        Ixz = -float(np.sum(rel[:, 0] * rel[:, 2] * m))
        Iyz = -float(np.sum(rel[:, 1] * rel[:, 2] * m))
        v = (rel - relp) / frame_length
        I = np.array([[Ixx, Ixy, Ixz], [Ixy, Iyy, Iyz], [Ixz, Iyz, Izz]])
        ev, E = np.linalg.eigh(I)
        rot = 0.0
        for j in range(3):
            e = E[:, j]
            dp = rel @ e
            rad = rel - dp[:, None] * e[None, :]
            L = np.array([np.sum(rad[:, 1] * v[:, 2] * m - rad[:, 2] * v[:, 1] * m),
                          np.sum(rad[:, 2] * v[:, 0] * m - rad[:, 0] * v[:, 2] * m),
                          np.sum(rad[:, 0] * v[:, 1] * m - rad[:, 1] * v[:, 0] * m)])
            rot += float(L @ L) / (2 * ev[j]) * conv
        ke = 0.5 * M * float(np.sum((p - c) ** 2)) / frame_length ** 2 * conv
        out.append((ke, rot))
        prev = x
    return np.array(out)


def nb_make_list(g, mask1, mask2, fep=False):
    """calc_nb.f90 nb_make_list (:334-759), pair by pair in the reference's
    loop order (every mask-1 atom, then every mask-2 atom, both ascending).

    A pair is dropped when
      * atom1 >= atom2 and atom2 is in both masks (:401-410; the pairs inside
        the overlap are taken once, and also any pair whose second atom is in
        the overlap and whose first atom has the larger index);
      * the two atoms share an angle of the topology (:412-425).
    LJ code: the topology's type pair code (1, or 2 for the polar pairs),
    3 for a 1-4 pair (:442-461).  Per state s (one state without fep):
      geometric rule  AA = a1*a2, BB = b1*b2;  arithmetic rule AA = a1 + a2,
      BB = b1*b2, with a, b the atom's parameters at the LJ code; a Q atom
      (a solute atom with a Q index, fep only) takes its state's Q type and,
      for code 2 with a non-Q partner, its code-1 value (:463-683);
      charge product: fep q1*q2*(el14 scale if 1-4 else 1), Q atoms at their
      state's charge (:684-740); without fep crg1*crg2*el14_scale for every
      pair (:742, as the reference has it).
    The charges of g carry sqrt(Coulomb constant), so the products are the
    reference's charge product times the constant.
    Returns (pairs [n, 2], AA [n, S], BB [n, S], qq [n, S])."""
    natom, nsol = int(g.natom), int(g.nat_solute)
    in1 = np.zeros(natom, bool); in1[np.asarray(mask1, dtype=np.int64)] = True
    in2 = np.zeros(natom, bool); in2[np.asarray(mask2, dtype=np.int64)] = True
    group1 = [j for j in range(natom) if in1[j]]
    group2 = [k for k in range(natom) if in2[k]]
    mutual = set(j for j in group1 if in2[j])
    angles = [tuple(int(v) for v in a[:3]) for a in np.asarray(g.ang).reshape(len(g.ang), -1)] \
        if len(g.ang) else []
    p14 = set(tuple(sorted((int(a), int(b)))) for a, b in np.asarray(g.pairs14).reshape(-1, 2))
    iac = np.asarray(g.iac)
    avdw, bvdw = np.asarray(g.avdw), np.asarray(g.bvdw)
    ljcod = np.asarray(g.ljcod)
    crg = np.asarray(g.crg)
    S = int(g.nstates) if fep else 1
    iqatom = np.asarray(g.iqatom)
    qiac, qcrg = np.asarray(g.qiac), np.asarray(g.qcrg)
    qavdw, qbvdw = np.asarray(g.qavdw), np.asarray(g.qbvdw)
    arith = int(getattr(g, "ivdw_rule", 1)) == 2
    el14 = float(g.el14_scale)

    def is_q(a):
        return fep and a < nsol and iqatom[a] >= 0

    pairs, AA, BB, QQ = [], [], [], []
    for j in group1:
        for k in group2:
            if j >= k and k in mutual:
                continue
            if any((a == j and (b == k or c == k)) or (b == j and (a == k or c == k)) or
                   (c == j and (a == k or b == k)) for a, b, c in angles):
                continue
            code = int(ljcod[iac[j], iac[k]])
            if (min(j, k), max(j, k)) in p14:
                code = 3
            aa, bb, qq = [], [], []
            for s in range(S):
                par = []
                for me, other in ((j, k), (k, j)):
                    if is_q(me):
                        c = 1 if (code == 2 and not is_q(other)) else code
                        t = qiac[iqatom[me], s]
                        par.append((qavdw[t, c - 1], qbvdw[t, c - 1], qcrg[iqatom[me], s]))
                    else:
                        par.append((avdw[iac[me], code - 1], bvdw[iac[me], code - 1], crg[me]))
                (a1, b1, q1), (a2, b2, q2) = par
                aa.append(a1 + a2 if arith else a1 * a2)
                bb.append(b1 * b2)
                if fep:
                    qq.append(q1 * q2 * el14 if code == 3 else q1 * q2)
                else:
                    qq.append(q1 * q2 * el14)
            pairs.append((j, k)); AA.append(aa); BB.append(bb); QQ.append(qq)
    f = lambda v: np.array(v, dtype=np.float64).reshape(-1, S)
    return np.array(pairs, dtype=np.int64).reshape(-1, 2), f(AA), f(BB), f(QQ)


def nb_calc(frames, pairs, AA, BB, qq, lambdas=None, arith=False):
    """calc_nb.f90 nb_calc_lists (:257-328): per frame, pair by pair in list
    order, r = sqrt(dx**2 + dy**2 + dz**2); a pair at r = 0 adds nothing;
    invr6 = invr**6 (six products), invr12 = invr6**2;
      geometric  Vlj += lam_s*(AA*invr12 - BB*invr6)
      arithmetic Vlj += lam_s*(sqrt(BB)*AA**6*invr6*(AA**6*invr6 - 2))
      Vel += lam_s*qq*invr
    over the states s (lam = 1 and one state without fep).
    Returns [nframes, 2] (Vlj, Vel)."""
    S = AA.shape[1]
    lam = [1.0] if lambdas is None else [float(v) for v in lambdas]
    out = []
    for fr in np.asarray(frames, dtype=np.float64):
        x = fr.reshape(-1, 3)
        vlj = vel = 0.0
        for p in range(len(pairs)):
            j, k = int(pairs[p, 0]), int(pairs[p, 1])
            r = math.sqrt((x[j, 0] - x[k, 0]) ** 2 + (x[j, 1] - x[k, 1]) ** 2 + (x[j, 2] - x[k, 2]) ** 2)
            if r == 0:
                continue
            invr = 1.0 / r
            invr6 = invr * invr * invr * invr * invr * invr
            invr12 = invr6 * invr6
            for s in range(S):
                a, b = float(AA[p, s]), float(BB[p, s])
                if arith:
                    a6 = a ** 6
                    vlj += lam[s] * (math.sqrt(b) * a6 * invr6 * (a6 * invr6 - 2.0))
                else:
                    vlj += lam[s] * (a * invr12 - b * invr6)
                vel += lam[s] * (float(qq[p, s]) * invr)
        out.append((vlj, vel))
    return np.array(out, dtype=np.float64).reshape(-1, 2)


def nb_qp(frames, g, residues, qmask, fep=False, lambdas=None):
    """calc_nb.f90 nb_qp_add / nb_qp_calc (:778-959): per residue the list of
    its atoms against the Q-atom mask (nb_make_list), and per frame each
    residue's nb_calc_lists.  Returns [nframes, nresidues, 2]."""
    out = []
    for r in residues:
        p, A, B, Q = nb_make_list(g, r, qmask, fep=fep)
        out.append(nb_calc(frames, p, A, B, Q, lambdas=lambdas, arith=int(getattr(g, "ivdw_rule", 1)) == 2))
    return np.stack(out, 1)


def nb_averages(values):
    """calc_nb.f90 nb_calc (:248-251): the running averages
    ave = (ave*n + V)/(n + 1) after each frame; returns the last."""
    ave, n = 0.0, 0
    for v in values:
        ave = (ave * n + float(v)) / (n + 1)
        n += 1
    return ave
