"""CPU restatement of qfep's Parts 1-3 (TEST INFRASTRUCTURE; parity unpinned by
reference data for Parts 2-3: the reference ships no EVB mapping output).

Only the tests load this file, as the checker of qgpu_qfep_evb.  It follows
src/qfep.f90 of the reference (qusers/qsource, Q 5.06) statement by
statement in plain Python/numpy, with its own reader of the energy files
(get_ene, src/nrgy.f90:147-188):
  file loop, alpha shift, Hij and ground state   :416-530 (more than two
      states: the lowest eigenvalue by numpy.linalg.eigvalsh, where qfep
      uses tred2/tqli)
  Part 1 (dGf, dGr, dG)                           :609-661
  Part 2 (bins of the gap, diabatic and ground-state free energies)
                                                  :712-812
  Part 3 (bin averages over windows; min over all bins incl. empty ones)
                                                  :814-835
The reference ships no EVB mapping data with its restart files, so the pin
is this line-by-line restatement run on the same files.
"""
import math
import struct

import numpy as np


def _records(path):
    data = open(path, "rb").read()
    k = 0
    while k + 4 <= len(data):
        (n,) = struct.unpack_from("<i", data, k)
        yield data[k + 4:k + 4 + n]
        k += 8 + n


def read_en(path, nstates, num_offd, gas=False):
    recs = list(_records(path))
    assert struct.unpack_from("<i", recs[0])[0] == 1337
    lam, frames = None, []
    k = 1
    while k + nstates < len(recs):   # nstates state records and the OFFD record
        E, L = [], []
        for s in range(nstates):
            v = struct.unpack_from("<15d", recs[k + s], 4)
            L.append(v[0])
            # total, or q bond + angle + torsion + improper + qq el + qq vdW + restraint
            E.append(((((((v[2] + v[3]) + v[4]) + v[5]) + v[8]) + v[9]) + v[14]) if gas else v[1])
        off = recs[k + nstates]
        od = [struct.unpack_from("<2i2d", off, 24 * c) for c in range(num_offd)]
        if lam is None:
            lam = L
        frames.append((E, od))
        k += nstates + 1
    return lam, frames


def evb(paths, nstates, kT, noffd=0, nskip=0, gas=False, nbins=20, nmin=1, alpha=None, scale_hij=0.0,
        couplings=(), coeff=None):
    """qfep Parts 1-3 on energy files (one per window, in lambda order)."""
    num_offd = noffd if noffd != 0 else len(couplings)
    windows = [read_en(p, nstates, num_offd, gas) for p in paths]
    return evb_windows(windows, nstates, kT, noffd, nskip, nbins, nmin, alpha, scale_hij, couplings, coeff)


def evb_windows(windows, nstates, kT, noffd=0, nskip=0, nbins=20, nmin=1, alpha=None, scale_hij=0.0,
                couplings=(), coeff=None):
    """qfep Parts 1-3 on windows given as (lambdas, frames), each frame
    (per-state energies, [(i, j, Hij, rkl) per coupling]) as read_en returns
    them."""
    S = nstates
    rt = kT
    num_offd = noffd if noffd != 0 else len(couplings)
    alfa = [0.0] + [alpha[i] if alpha and i < len(alpha) else 0.0 for i in range(1, S)]   # alfa(1) = 0
    cf = list(coeff) if coeff is not None else [-1.0, 1.0] + [0.0] * (S - 2)
    A = np.zeros((S, S)); mu = np.zeros((S, S)); eta = np.zeros((S, S)); r0 = np.zeros((S, S))
    if noffd == 0:
        for (i, j, a, m, e, r) in couplings:
            A[i - 1, j - 1], mu[i - 1, j - 1], eta[i - 1, j - 1], r0[i - 1, j - 1] = a, m, e, r
    gapmin, gapmax = 999.0, -999.0
    F = []
    for lam, frames in windows:
        v, vg, c1, c2, gap, rr = [], [], [], [], [], []
        for ipt, (E, od) in enumerate(frames, start=1):
            E = [E[i] + alfa[i] for i in range(S)]
            H = np.zeros((S, S))
            if scale_hij > 0:
                h12 = 0.0
                for (i, j, hij, rkl) in od[:noffd]:
                    if (i, j) == (1, 2):
                        h12 = hij
                H[0, 1] = scale_hij * h12
            else:
                r1 = od[0][3] if num_offd > 0 else 0.0
                for i in range(S):
                    for j in range(S):
                        if i == j:
                            H[i, j] = E[i]
                        elif A[i, j] == 0.0:
                            H[i, j] = A[j, i] * math.exp(-mu[j, i] * (r1 - r0[j, i])) * \
                                math.exp(-eta[j, i] * (r1 - r0[j, i]) ** 2)
                        else:
                            H[i, j] = A[i, j] * math.exp(-mu[i, j] * (r1 - r0[i, j])) * \
                                math.exp(-eta[i, j] * (r1 - r0[i, j]) ** 2)
            a1 = b1 = 0.0
            if S == 2:
                g = 0.5 * (E[0] + E[1]) - 0.5 * math.sqrt((E[0] - E[1]) ** 2 + 4.0 * H[0, 1] ** 2)
                if num_offd > 0:
                    a1 = 1.0 / (1.0 + ((g - E[0]) / H[0, 1]) ** 2)
                    b1 = 1.0 - a1
            else:
                g = float(np.linalg.eigvalsh(H)[0])
            gp = 0.0
            for i in range(S):
                gp = gp + E[i] * cf[i]
            if ipt > nskip:
                if gp < gapmin:
                    gapmin = gp
                if gp > gapmax:
                    gapmax = gp
            v.append(E); vg.append(g); c1.append(a1); c2.append(b1); gap.append(gp)
            rr.append(od[0][3] if num_offd > 0 else 0.0)
        F.append(dict(lam=lam, v=v, vg=vg, c1=c1, c2=c2, gap=gap, r=rr, npts=len(frames)))
    n = len(F)

    def zw(f, g):
        s = 0.0
        for ipt in range(nskip, f["npts"]):
            v1 = v2 = 0.0
            for i in range(S):
                v1 = v1 + f["lam"][i] * f["v"][ipt][i]
                v2 = v2 + g["lam"][i] * f["v"][ipt][i]
            s = s + math.exp(-(v2 - v1) / rt)
        return -rt * math.log(s / (f["npts"] - nskip))
    dgf = [zw(F[w], F[w + 1]) for w in range(n - 1)] + [0.0]
    dgr = [0.0] + [zw(F[w], F[w - 1]) for w in range(1, n)]
    dG = [0.0]
    for w in range(1, n):
        dG.append(dG[-1] + 0.5 * (dgf[w - 1] - dgr[w]))
    part1 = np.array([[dgf[w], dgr[w], dG[w]] for w in range(n)])
    xint = (gapmax - gapmin) / nbins
    MB = nbins + 1
    bs = np.zeros((MB, 4)); ptsum = np.zeros(MB)
    part2 = np.zeros((n, nbins, 5 + S))
    for w, f in enumerate(F):
        avdvv = np.zeros((S, MB)); avdvg = np.zeros(MB); avc1 = np.zeros(MB); avc2 = np.zeros(MB); avr = np.zeros(MB)
        sumv = np.zeros((S, MB)); sumg = np.zeros(MB); nbp = np.zeros(MB, dtype=int)
        binof = [int((f["gap"][i] - gapmin) / xint) for i in range(f["npts"])]
        for ipt in range(nskip, f["npts"]):
            b = binof[ipt]
            ve = 0.0
            for i in range(S):
                ve = ve + f["lam"][i] * f["v"][ipt][i]
            for i in range(S):
                avdvv[i, b] += f["v"][ipt][i] - ve
            avdvg[b] += f["vg"][ipt] - ve
            avc1[b] += f["c1"][ipt]; avc2[b] += f["c2"][ipt]
            if num_offd > 0:
                avr[b] += f["r"][ipt]
            nbp[b] += 1
        for b in range(nbins):
            if nbp[b]:
                avc1[b] /= nbp[b]; avc2[b] /= nbp[b]; avr[b] /= nbp[b]
                avdvv[:, b] /= nbp[b]; avdvg[b] /= nbp[b]
        for ipt in range(nskip, f["npts"]):
            b = binof[ipt]
            ve = 0.0
            for i in range(S):
                ve = ve + f["lam"][i] * f["v"][ipt][i]
            for i in range(S):
                sumv[i, b] += math.exp(-(f["v"][ipt][i] - ve - avdvv[i, b]) / rt)
            sumg[b] += math.exp(-(f["vg"][ipt] - ve - avdvg[b]) / rt)
        for b in range(nbins):
            part2[w, b, 0] = nbp[b]
            if nbp[b] < nmin:
                continue
            bs[b, 1] += avc1[b] * nbp[b]; bs[b, 2] += avc2[b] * nbp[b]; bs[b, 3] += avr[b] * nbp[b]
            ptsum[b] += nbp[b]
            dGg = dG[w] + (-rt * math.log(sumg[b] / nbp[b]) + avdvg[b])
            bs[b, 0] += dGg * nbp[b]
            part2[w, b, 1:5] = [gapmin + (b + 1) * xint - xint / 2.0, dGg, avc1[b], avc2[b]]
            for i in range(S):
                part2[w, b, 5 + i] = dG[w] + (-rt * math.log(sumv[i, b] / nbp[b]) + avdvv[i, b])
    for b in range(nbins):
        if ptsum[b] >= nmin:
            bs[b] /= ptsum[b]
    mn = bs[:, 0].min()
    part3 = np.zeros((nbins, 7))
    for b in range(nbins):
        part3[b, 0] = ptsum[b]
        if ptsum[b] >= nmin:
            part3[b, 1:] = [gapmin + (b + 1) * xint - xint / 2.0, bs[b, 0], bs[b, 0] - mn, bs[b, 1], bs[b, 2], bs[b, 3]]
    return {"part1": part1, "gap": np.array([gapmin, gapmax]), "part2": part2, "part3": part3,
            "npts": np.array([f["npts"] for f in F])}
