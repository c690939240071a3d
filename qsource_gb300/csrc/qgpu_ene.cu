// qgpu_ene.cu -- Q energy files (.en), the binary file qfep reads.
//
// Layout (Fortran unformatted sequential records, each framed by a 4-byte
// length before and after the payload, as gfortran writes them):
//   header (prep_sim_version, src/md.f90:17011-17015), arrays = 1:
//     int32 canary (1337 = double precision), arrays (1), totresid (1),
//     types(1) (NOGC = 3, misc.f90:36), numres(1) (1), resid(1) (-1),
//     gcnum(1) (-1), char[80] version
//   per frame (put_ene, src/nrgy.f90:94-123):
//     nstates records: int32 state (1-based), f64 lambda, total, q%bond,
//       q%angle, q%torsion, q%improper, qx%el, qx%vdw, qq%el, qq%vdw, qp%el,
//       qp%vdw, qw%el, qw%vdw, restraint
//     one OFFD record: per coupling int32 i, int32 j, f64 Hij, f64 rkl (empty
//       when there are none)
// qdyn writes a frame at every nonzero multiple of iene_cycle
// (md_run, src/md.f90:6630-6633).  Host code only.
#include <stdio.h>
#include <string.h>

#include <cmath>

#include <vector>

#include "qgpu_internal.cuh"

namespace {

bool put_record(FILE *f, const void *payload, int32_t n) {
    return fwrite(&n, 4, 1, f) == 1 && (n == 0 || fwrite(payload, 1, (size_t)n, f) == (size_t)n) &&
           fwrite(&n, 4, 1, f) == 1;
}

struct Rec {
    std::vector<unsigned char> b;
    void i32(int32_t v) { const unsigned char *p = (const unsigned char *)&v; b.insert(b.end(), p, p + 4); }
    void f64(double v) { const unsigned char *p = (const unsigned char *)&v; b.insert(b.end(), p, p + 8); }
};

}  // namespace

// header record; returns 0 or QGPU_E_INVALID
int qgpu_ene_write_header(FILE *f, const char *version) {
    Rec r;
    r.i32(1337); r.i32(1); r.i32(1); r.i32(3); r.i32(1); r.i32(-1); r.i32(-1);
    char v[80];
    memset(v, ' ', sizeof v);
    const char *src = version ? version : "";
    memcpy(v, src, strnlen(src, sizeof v));
    r.b.insert(r.b.end(), v, v + 80);
    return put_record(f, r.b.data(), (int32_t)r.b.size()) ? 0 : QGPU_E_INVALID;
}

// one frame: nstates state records and the OFFD record
int qgpu_ene_write_frame(FILE *f, int32_t nstates, const qgpu_qenergy *EQ, int32_t noffd, const int32_t *offd_ij,
                         const double *offd_Hr) {
    for (int s = 0; s < nstates; ++s) {
        const qgpu_qenergy &q = EQ[s];
        Rec r;
        r.i32(s + 1);
        const double v[15] = {q.lambda, q.total, q.q_bond, q.q_angle, q.q_torsion, q.q_improper, q.qx_el, q.qx_vdw,
                              q.qq_el, q.qq_vdw, q.qp_el, q.qp_vdw, q.qw_el, q.qw_vdw, q.restraint};
        for (double x : v) r.f64(x);
        if (!put_record(f, r.b.data(), (int32_t)r.b.size())) return QGPU_E_INVALID;
    }
    Rec o;
    for (int k = 0; k < noffd; ++k) {
        o.i32(offd_ij[2 * k]); o.i32(offd_ij[2 * k + 1]);
        o.f64(offd_Hr[2 * k]); o.f64(offd_Hr[2 * k + 1]);
    }
    return put_record(f, o.b.data(), (int32_t)o.b.size()) ? 0 : QGPU_E_INVALID;
}

extern "C" int qgpu_enefile_write(const char *path, int32_t nframes, int32_t nstates, const qgpu_qenergy *frames,
                                  int32_t noffd, const int32_t *offd_ij, const double *offd_Hr) {
    if (!path || nframes < 0 || nstates < 1 || nstates > QGPU_MAX_STATES || (nframes && !frames) || noffd < 0 ||
        (noffd && (!offd_ij || !offd_Hr)))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_enefile_write: bad arguments");
    FILE *f = fopen(path, "wb");
    if (!f) return qgpu_fail(QGPU_E_INVALID, "qgpu_enefile_write: cannot open %s", path);
    int rc = qgpu_ene_write_header(f, "5.06 (qsource_gb300)");
    for (int k = 0; k < nframes && !rc; ++k)
        rc = qgpu_ene_write_frame(f, nstates, frames + (size_t)k * nstates, noffd, offd_ij,
                                  offd_Hr ? offd_Hr + (size_t)k * 2 * noffd : nullptr);
    if (fclose(f) != 0 && !rc) rc = QGPU_E_INVALID;
    if (rc) return qgpu_fail(rc, "qgpu_enefile_write: write to %s failed", path);
    return 0;
}

// ---------------------------------------------------------------- qfep EVB
// qfep Parts 1-3 (src/qfep.f90:416-835) over energy files, host code.
namespace {

long get_record(FILE *f, std::vector<unsigned char> &buf) {
    int32_t n, m;
    if (fread(&n, 4, 1, f) != 1) return -1;
    if (n < 0) return -2;
    buf.resize((size_t)n);
    if (n && fread(buf.data(), 1, (size_t)n, f) != (size_t)n) return -2;
    if (fread(&m, 4, 1, f) != 1 || m != n) return -2;
    return n;
}
double f64_at(const std::vector<unsigned char> &b, size_t off) {
    double v;
    memcpy(&v, b.data() + off, 8);
    return v;
}
int32_t i32_at(const std::vector<unsigned char> &b, size_t off) {
    int32_t v;
    memcpy(&v, b.data() + off, 4);
    return v;
}

// One window's frames: shifted state energies, ground state, mixing, gap and
// the first coupling's distance per frame.
struct EvbWindow {
    std::vector<double> lam, v, vg, c1, c2, gap, r;
    int npts = 0;
};

// Lowest eigenvalue of a symmetric n x n matrix (row-major) by cyclic Jacobi
// rotations (each rotation zeroes one off-diagonal element; the diagonal
// converges to the eigenvalues).
double lowest_eigenvalue(std::vector<double> a, int n) {
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i) {
            diag += a[i * n + i] * a[i * n + i];
            for (int j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
        }
        if (off <= 1e-30 * (diag + 1e-300)) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[p * n + q];
                if (apq == 0.0) continue;
                const double th = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                const double t = std::fabs(th) > 1e150 ? 0.5 / th
                                                       : (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
            }
    }
    double m = a[0];
    for (int i = 1; i < n; ++i) m = std::fmin(m, a[i * n + i]);
    return m;
}

// Reads one energy file and forms the per-frame EVB quantities (the file loop
// of qfep, src/qfep.f90:247-530).  Returns false on an unreadable file.
bool evb_read(const char *path, const qgpu_qfep_params &p, int num_offd, const std::vector<double> &A,
              const std::vector<double> &mu, const std::vector<double> &eta, const std::vector<double> &r0,
              EvbWindow &W, double &gapmin, double &gapmax) {
    const int S = p.nstates;
    FILE *f = fopen(path, "rb");
    if (!f) return false;
    std::vector<unsigned char> b;
    const long nh = get_record(f, b);
    if (nh < 8 || i32_at(b, 0) != 1337 || i32_at(b, 4) != 1) { fclose(f); return false; }
    std::vector<double> E(S), H((size_t)S * S);
    std::vector<int32_t> oi(num_offd), oj(num_offd);
    std::vector<double> oH(num_offd), orr(num_offd);
    bool ok = true;
    for (;;) {
        int s = 0;
        for (; s < S; ++s) {
            if (get_record(f, b) < 4 + 8 * 15) break;
            if (W.npts == 0) W.lam.push_back(f64_at(b, 4));
            // record: state, lambda, total, q bond/angle/torsion/improper,
            // qx, qq, qp, qw (el, vdW), restraint
            E[s] = p.gas ? f64_at(b, 20) + f64_at(b, 28) + f64_at(b, 36) + f64_at(b, 44) + f64_at(b, 68) +
                               f64_at(b, 76) + f64_at(b, 116)
                         : f64_at(b, 12);
        }
        if (s < S) break;
        const long no = get_record(f, b);
        if (no < 0) break;
        if (no < 24L * num_offd) { ok = false; break; }
        for (int k = 0; k < num_offd; ++k) {
            oi[k] = i32_at(b, 24 * k); oj[k] = i32_at(b, 24 * k + 4);
            oH[k] = f64_at(b, 24 * k + 8); orr[k] = f64_at(b, 24 * k + 16);
        }
        for (int i = 1; i < S; ++i) E[i] += p.alpha[i];
        // off-diagonal elements (src/qfep.f90:463-495)
        double h12 = 0.0;
        if (p.scale_hij > 0.0) {
            for (int k = 0; k < p.noffd && k < num_offd; ++k)
                if (oi[k] == 1 && oj[k] == 2) h12 = oH[k];
            h12 *= p.scale_hij;
        } else {
            const double r1 = num_offd > 0 ? orr[0] : 0.0;
            for (int i = 0; i < S; ++i)
                for (int j = 0; j < S; ++j) {
                    if (i == j) { H[i * S + j] = E[i]; continue; }
                    const int e = A[i * S + j] == 0.0 ? j * S + i : i * S + j;
                    const double dr = r1 - r0[e];
                    H[i * S + j] = A[e] * std::exp(-mu[e] * dr) * std::exp(-eta[e] * dr * dr);
                }
            if (S > 1) h12 = H[1];
        }
        // ground state (src/qfep.f90:500-513)
        double vg, c1 = 0.0, c2 = 0.0;
        if (S == 2) {
            vg = 0.5 * (E[0] + E[1]) - 0.5 * std::sqrt((E[0] - E[1]) * (E[0] - E[1]) + 4.0 * h12 * h12);
            if (num_offd > 0) {
                const double x = (vg - E[0]) / h12;
                c1 = 1.0 / (1.0 + x * x);
                c2 = 1.0 - c1;
            }
        } else {
            vg = lowest_eigenvalue(H, S);
        }
        double gap = 0.0;
        for (int i = 0; i < S; ++i) gap = gap + E[i] * p.coeff[i];
        W.npts++;
        if (W.npts > p.nskip) {
            if (gap < gapmin) gapmin = gap;
            if (gap > gapmax) gapmax = gap;
        }
        W.v.insert(W.v.end(), E.begin(), E.end());
        W.vg.push_back(vg); W.c1.push_back(c1); W.c2.push_back(c2); W.gap.push_back(gap);
        W.r.push_back(num_offd > 0 ? orr[0] : 0.0);
    }
    fclose(f);
    return ok;
}

}  // namespace

extern "C" int qgpu_qfep_evb(int32_t nfiles, const char *const *paths, const qgpu_qfep_params *p, double *part1,
                             double *gaprange, double *part2, double *part3, int32_t *npts) {
    if (nfiles < 2 || !paths || !p || !part1 || !gaprange || !part2 || !part3 || !npts)
        return qgpu_fail(QGPU_E_INVALID, "qgpu_qfep_evb: bad arguments (at least two files)");
    const int S = p->nstates, NB = p->nbins;
    if (S < 1 || S > QGPU_MAX_STATES || p->noffd < 0 || NB < 1 || p->nmin < 1 || !(p->kT > 0.0) || p->nskip < 0 ||
        p->ncoup < 0 || p->ncoup > QGPU_QFEP_MAXCOUP || (p->scale_hij > 0.0 && S != 2))
        return qgpu_fail(QGPU_E_INVALID, "qgpu_qfep_evb: bad parameters");
    const int num_offd = p->noffd != 0 ? p->noffd : p->ncoup;
    std::vector<double> A((size_t)S * S, 0.0), mu(A), eta(A), r0(A);
    if (p->noffd == 0)
        for (int c = 0; c < p->ncoup; ++c) {
            const int i = p->coup_ij[2 * c] - 1, j = p->coup_ij[2 * c + 1] - 1;
            if (i < 0 || j < 0 || i >= S || j >= S || i == j)
                return qgpu_fail(QGPU_E_INVALID, "qgpu_qfep_evb: coupling %d names states %d, %d", c, i + 1, j + 1);
            A[i * S + j] = p->coup_A[c]; mu[i * S + j] = p->coup_mu[c];
            eta[i * S + j] = p->coup_eta[c]; r0[i * S + j] = p->coup_rxy0[c];
        }
    std::vector<EvbWindow> W(nfiles);
    double gapmin = 999.0, gapmax = -999.0;   // qfep's starting values
    for (int w = 0; w < nfiles; ++w) {
        if (!paths[w] || !evb_read(paths[w], *p, num_offd, A, mu, eta, r0, W[w], gapmin, gapmax))
            return qgpu_fail(QGPU_E_INVALID, "qgpu_qfep_evb: cannot read energy file %s", paths[w] ? paths[w] : "(null)");
        npts[w] = W[w].npts;
        if (W[w].npts <= p->nskip)
            return qgpu_fail(QGPU_E_INVALID, "qgpu_qfep_evb: %s has no frames after the %d skipped", paths[w], p->nskip);
    }
    const double rt = p->kT;
    // Part 1 (src/qfep.f90:609-661)
    std::vector<double> dgf(nfiles + 1, 0.0), dgr(nfiles + 1, 0.0), dG(nfiles, 0.0);
    auto zwanzig = [&](const EvbWindow &F, const EvbWindow &G) {
        double sum = 0.0;
        for (int q = p->nskip; q < F.npts; ++q) {
            double v1 = 0.0, v2 = 0.0;
            for (int s = 0; s < S; ++s) {
                v1 = v1 + F.lam[s] * F.v[(size_t)q * S + s];
                v2 = v2 + G.lam[s] * F.v[(size_t)q * S + s];
            }
            sum = sum + std::exp(-(v2 - v1) / rt);
        }
        return -rt * std::log(sum / (double)(F.npts - p->nskip));
    };
    for (int w = 0; w + 1 < nfiles; ++w) dgf[w] = zwanzig(W[w], W[w + 1]);
    for (int w = nfiles - 1; w >= 1; --w) dgr[w] = zwanzig(W[w], W[w - 1]);
    for (int w = 1; w < nfiles; ++w) dG[w] = dG[w - 1] + 0.5 * (dgf[w - 1] - dgr[w]);
    for (int w = 0; w < nfiles; ++w) {
        part1[3 * w] = w + 1 < nfiles ? dgf[w] : 0.0;
        part1[3 * w + 1] = w > 0 ? dgr[w] : 0.0;
        part1[3 * w + 2] = dG[w];
    }
    gaprange[0] = gapmin; gaprange[1] = gapmax;
    const double xint = (gapmax - gapmin) / (double)(float)NB;
    if (!(xint > 0.0)) return qgpu_fail(QGPU_E_INVALID, "qgpu_qfep_evb: the energy gap does not vary");
    // Part 2 (src/qfep.f90:712-812); bins 1..NB+1 (the largest gap falls in NB+1)
    const int MB = NB + 1;
    std::vector<double> bs1(MB, 0.0), bs2(MB, 0.0), bs3(MB, 0.0), bs4(MB, 0.0), ptsum(MB, 0.0);
    memset(part2, 0, sizeof(double) * (size_t)nfiles * NB * QGPU_QFEP_P2);
    memset(part3, 0, sizeof(double) * (size_t)NB * QGPU_QFEP_P3);
    for (int w = 0; w < nfiles; ++w) {
        const EvbWindow &F = W[w];
        std::vector<double> avdvv((size_t)S * MB, 0.0), avdvg(MB, 0.0), avc1(MB, 0.0), avc2(MB, 0.0), avr(MB, 0.0);
        std::vector<double> sumv((size_t)S * MB, 0.0), sumg(MB, 0.0);
        std::vector<int> nbp(MB, 0);
        auto bin_of = [&](int q) {
            const int b = (int)((F.gap[q] - gapmin) / xint);
            return b < 0 ? 0 : (b > NB ? NB : b);   // 0-based; NB is qfep's bin NB+1
        };
        auto veff_of = [&](int q) {
            double ve = 0.0;
            for (int s = 0; s < S; ++s) ve = ve + F.lam[s] * F.v[(size_t)q * S + s];
            return ve;
        };
        for (int q = p->nskip; q < F.npts; ++q) {
            const int b = bin_of(q);
            const double ve = veff_of(q);
            for (int s = 0; s < S; ++s) avdvv[(size_t)s * MB + b] += F.v[(size_t)q * S + s] - ve;
            avdvg[b] += F.vg[q] - ve;
            avc1[b] += F.c1[q];
            avc2[b] += F.c2[q];
            if (num_offd > 0) avr[b] += F.r[q];
            nbp[b]++;
        }
        for (int b = 0; b < NB; ++b)
            if (nbp[b] != 0) {
                const double n = (double)nbp[b];
                avc1[b] /= n; avc2[b] /= n; avr[b] /= n;
                for (int s = 0; s < S; ++s) avdvv[(size_t)s * MB + b] /= n;
                avdvg[b] /= n;
            }
        for (int q = p->nskip; q < F.npts; ++q) {
            const int b = bin_of(q);
            const double ve = veff_of(q);
            for (int s = 0; s < S; ++s)
                sumv[(size_t)s * MB + b] += std::exp(-(F.v[(size_t)q * S + s] - ve - avdvv[(size_t)s * MB + b]) / rt);
            sumg[b] += std::exp(-(F.vg[q] - ve - avdvg[b]) / rt);
        }
        for (int b = 0; b < NB; ++b) {
            double *row = part2 + ((size_t)w * NB + b) * QGPU_QFEP_P2;
            row[0] = nbp[b];
            if (nbp[b] < p->nmin) continue;
            const double n = (double)nbp[b];
            bs2[b] += avc1[b] * n;
            bs3[b] += avc2[b] * n;
            bs4[b] += avr[b] * n;
            ptsum[b] += n;
            const double dGg = dG[w] + (-rt * std::log(sumg[b] / n) + avdvg[b]);
            bs1[b] += dGg * n;
            row[1] = gapmin + (double)(b + 1) * xint - xint / 2.0;
            row[2] = dGg;
            row[3] = avc1[b];
            row[4] = avc2[b];
            for (int s = 0; s < S; ++s)
                row[5 + s] = dG[w] + (-rt * std::log(sumv[(size_t)s * MB + b] / n) + avdvv[(size_t)s * MB + b]);
        }
    }
    // Part 3 (src/qfep.f90:814-835)
    for (int b = 0; b < NB; ++b)
        if (ptsum[b] >= p->nmin) { bs1[b] /= ptsum[b]; bs2[b] /= ptsum[b]; bs3[b] /= ptsum[b]; bs4[b] /= ptsum[b]; }
    double mn = bs1[0];
    for (int b = 1; b < MB; ++b) mn = std::fmin(mn, bs1[b]);
    for (int b = 0; b < NB; ++b) {
        double *row = part3 + (size_t)b * QGPU_QFEP_P3;
        row[0] = ptsum[b];
        if (ptsum[b] < p->nmin) continue;
        row[1] = gapmin + (double)(b + 1) * xint - xint / 2.0;
        row[2] = bs1[b]; row[3] = bs1[b] - mn; row[4] = bs2[b]; row[5] = bs3[b]; row[6] = bs4[b];
    }
    return 0;
}
