/*
 * qoracle.c -- FP64 CPU restatement of the qdyn hot path (TEST INFRASTRUCTURE).
 *
 * This file is the parity oracle for the GB300 engine.  It is not part of the
 * product: only the tests, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it, and only to check or time against it.
 *
 * It restates, in their serial (#else) branch semantics, the routines of the
 * reference qusers/qsource (Q 5.06) listed below.  Every list is built in the
 * reference's loop order (including the count-once parity rule), so list sets
 * can be compared exactly.  Compiled with -ffp-contract=off so that the FP64
 * cut-off tests round like a plain multiply/add sequence.
 *
 * Parity pin: tests/test_oracle_golden.py checks this file against the
 * reference's own step-0 golden energies (tests/basic_tests/SPH_*_benchmark.en
 * row 1, tests/test2/eval_test.sh:67, tests/test3/eval_test.sh:67).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#include "qgpu.h"

#define BOLTZ 0.001986          /* src/md.f90:54 */
#define SHAKE_TOL 0.0001        /* src/md.f90:460 */
#define SHAKE_MAX_ITER 1000     /* src/md.f90:461 */
#define QREAL_EPS 1.0e-14       /* src/sizes.f90:48 (double build) */
#define NLRF 43                 /* cent[3] phi0 phi1[3] phi2[9] phi3[27] */

/* si, sj: the atoms whose difference x[sj] - x[si] gives the periodic shift
   of the pair in a box (the switch atoms of the charge-group pair, the two
   water O, the Q switching atom and a solute / water atom); -1 in a sphere */
typedef struct { int32_t i, j; int8_t lj, qlj; int32_t si, sj; } nbrec;

typedef struct { nbrec *a; int64_t n, cap; } nblist;

typedef struct oracle {
    qgpu_system_desc d;
    int N, S;
    double *x, *v, *xx, *f, *winv;
    int32_t *iwhich;            /* atom -> charge group */
    double *lrf;                /* ncgp * NLRF */
    nblist pp, pw, ww, qp, qw;
    int qp_done, qw_done;
    /* exclusion / 1-4 lookup: per solute atom sorted partner lists (j > i) */
    int32_t *ex_first, *ex_j, *p14_first, *p14_j;
    qgpu_energies E;
    qgpu_qenergy EQ[QGPU_MAX_STATES];
    double Hij[QGPU_MAX_STATES][QGPU_MAX_STATES];
    double EMorseD[256];
    /* temperature state */
    double Temp, Tfree, Tfree_solute, Tfree_solvent, Tscale_solute, Tscale_solvent;
    int32_t irand, rand_new;
    int32_t iseed;              /* the argument the reference passes to randm */
    int status;
    int istep;                  /* md_run step counter (watpol's itdis_update) */
    /* water polarisation shells (wshell, src/md.f90:18185-18368) */
    double *theta_corr, *avtheta, *avn_insh;
    double *theta, *tdum, *theta0;
    int32_t *list_sh, *nsort, *n_insh;
    /* Langevin random-force amplitudes and Nose-Hoover chain */
    double *randva, *randfa;
    double xnh[64], vnh[64], qnh[64], Gnh[64];
    /* periodic box: 1/boxlength and the box centre put_back_in_box moves */
    double ibox[3], boxc[3];
    int32_t *istart_mol;
} oracle;

/* ------------------------------------------------------------------ utils */
static void *xmalloc(size_t n) { void *p = calloc(1, n ? n : 1); return p; }
static void *dupbuf(const void *src, size_t n) {
    void *p = xmalloc(n);
    if (src && n) memcpy(p, src, n);
    return p;
}
static void nb_push_s(nblist *l, int32_t i, int32_t j, int lj, int qlj, int32_t si, int32_t sj) {
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 1024;
        l->a = (nbrec *)realloc(l->a, (size_t)l->cap * sizeof(nbrec));
    }
    l->a[l->n].i = i; l->a[l->n].j = j; l->a[l->n].lj = (int8_t)lj; l->a[l->n].qlj = (int8_t)qlj;
    l->a[l->n].si = si; l->a[l->n].sj = sj;
    l->n++;
}
static inline int ljcod(const oracle *o, int ti, int tj) { return o->d.ljcod[ti * o->d.natyps + tj]; }
static inline double avdw(const oracle *o, int t, int c) { return o->d.avdw[t * 3 + c - 1]; }
static inline double bvdw(const oracle *o, int t, int c) { return o->d.bvdw[t * 3 + c - 1]; }
static inline int is_q(const oracle *o, int i) { return o->d.iqatom[i] >= 0; }
static inline double qcrg(const oracle *o, int iq, int s) { return o->d.qcrg[iq * o->S + s]; }

static int pair_in(const int32_t *first, const int32_t *js, int i, int j) {
    for (int k = first[i]; k < first[i + 1]; ++k) if (js[k] == j) return 1;
    return 0;
}
/* listex / listexlong lookup of src/md.f90:8116-8130 (pair stored once, i<j) */
static int excluded(const oracle *o, int i, int j) {
    if (i > j) { int t = i; i = j; j = t; }
    return pair_in(o->ex_first, o->ex_j, i, j);
}
/* list14 / list14long lookup of src/md.f90:8144-8166 */
static int is14(const oracle *o, int i, int j) {
    if (i > j) { int t = i; i = j; j = t; }
    return pair_in(o->p14_first, o->p14_j, i, j);
}
static void build_pair_csr(int n, int np, const int32_t *pairs, int32_t **first, int32_t **js) {
    int32_t *f = (int32_t *)xmalloc((size_t)(n + 1) * sizeof(int32_t));
    int32_t *j = (int32_t *)xmalloc((size_t)(np ? np : 1) * sizeof(int32_t));
    for (int k = 0; k < np; ++k) {
        int a = pairs[2 * k], b = pairs[2 * k + 1];
        int lo = a < b ? a : b;
        f[lo + 1]++;
    }
    for (int i = 0; i < n; ++i) f[i + 1] += f[i];
    int32_t *fill = (int32_t *)xmalloc((size_t)(n + 1) * sizeof(int32_t));
    memcpy(fill, f, (size_t)(n + 1) * sizeof(int32_t));
    for (int k = 0; k < np; ++k) {
        int a = pairs[2 * k], b = pairs[2 * k + 1];
        int lo = a < b ? a : b, hi = a < b ? b : a;
        j[fill[lo]++] = hi;
    }
    free(fill);
    *first = f; *js = j;
}

/* ---------------------------------------------------------------- create */
void *oracle_create(const qgpu_system_desc *in) {
    oracle *o = (oracle *)xmalloc(sizeof(oracle));
    o->d = *in;
    int N = in->natom;
    o->N = N; o->S = in->nstates;
    o->x = (double *)dupbuf(in->x, 3 * (size_t)N * sizeof(double));
    o->v = (double *)dupbuf(in->v, 3 * (size_t)N * sizeof(double));
    o->xx = (double *)xmalloc(3 * (size_t)N * sizeof(double));
    o->f = (double *)xmalloc(3 * (size_t)N * sizeof(double));
    o->winv = (double *)xmalloc((size_t)N * sizeof(double));
    /* winv = 1/mass (prep_sim, src/md.f90:16745) */
    for (int i = 0; i < N; ++i) o->winv[i] = 1.0 / in->mass[in->iac[i]];
    o->iwhich = (int32_t *)xmalloc((size_t)N * sizeof(int32_t));
    for (int g = 0; g < in->ncgp; ++g)
        for (int k = in->cgp_first[g]; k <= in->cgp_last[g]; ++k) o->iwhich[in->cgpatom[k]] = g;
    o->lrf = (double *)xmalloc((size_t)in->ncgp * NLRF * sizeof(double));
    build_pair_csr(N, in->nexcl, in->excl_pairs, &o->ex_first, &o->ex_j);
    build_pair_csr(N, in->n14, in->pairs14, &o->p14_first, &o->p14_j);
    for (int s = 0; s < o->S; ++s) o->EQ[s].lambda = in->lambda[s];
    o->Tscale_solute = o->Tscale_solvent = 1.0;
    /* copy the variable-length inputs the new terms keep referring to */
    o->d.rstseq_ij = (const int32_t *)dupbuf(in->rstseq_ij, 2 * (size_t)in->nrstr_seq * sizeof(int32_t));
    o->d.rstseq_fk = (const double *)dupbuf(in->rstseq_fk, (size_t)in->nrstr_seq * sizeof(double));
    o->d.rstseq_flags = (const int32_t *)dupbuf(in->rstseq_flags, 2 * (size_t)in->nrstr_seq * sizeof(int32_t));
    o->d.heavy = (const uint8_t *)dupbuf(in->heavy, in->heavy ? (size_t)N : 0);
    o->d.rstpos_i = (const int32_t *)dupbuf(in->rstpos_i, 2 * (size_t)in->nrstr_pos * sizeof(int32_t));
    o->d.rstpos_x = (const double *)dupbuf(in->rstpos_x, 6 * (size_t)in->nrstr_pos * sizeof(double));
    o->d.rstdis_i = (const int32_t *)dupbuf(in->rstdis_i, 3 * (size_t)in->nrstr_dist * sizeof(int32_t));
    o->d.rstdis_p = (const double *)dupbuf(in->rstdis_p, 3 * (size_t)in->nrstr_dist * sizeof(double));
    o->d.rstang_i = (const int32_t *)dupbuf(in->rstang_i, 4 * (size_t)in->nrstr_angl * sizeof(int32_t));
    o->d.rstang_p = (const double *)dupbuf(in->rstang_p, 2 * (size_t)in->nrstr_angl * sizeof(double));
    o->d.rstwal_i = (const int32_t *)dupbuf(in->rstwal_i, 3 * (size_t)in->nrstr_wall * sizeof(int32_t));
    o->d.rstwal_p = (const double *)dupbuf(in->rstwal_p, 4 * (size_t)in->nrstr_wall * sizeof(double));
    int ns = in->wpol_restr ? in->nwpolr_shell : 0;
    o->d.nwpolr_shell = ns;
    o->theta_corr = (double *)xmalloc((size_t)(ns + 1) * sizeof(double));
    o->avtheta = (double *)xmalloc((size_t)(ns + 1) * sizeof(double));
    o->avn_insh = (double *)xmalloc((size_t)(ns + 1) * sizeof(double));
    o->n_insh = (int32_t *)xmalloc((size_t)(ns + 1) * sizeof(int32_t));
    for (int k = 0; k < ns; ++k) o->theta_corr[k] = in->wshell_theta_corr ? in->wshell_theta_corr[k] : 0.0;
    int nw = (N - in->nat_solute) / 3;
    o->theta = (double *)xmalloc((size_t)(nw + 1) * sizeof(double));
    o->tdum = (double *)xmalloc((size_t)(nw + 1) * sizeof(double));
    o->theta0 = (double *)xmalloc((size_t)(nw + 1) * sizeof(double));
    o->list_sh = (int32_t *)xmalloc((size_t)(nw + 1) * (ns + 1) * sizeof(int32_t));
    o->nsort = (int32_t *)xmalloc((size_t)(nw + 1) * (ns + 1) * sizeof(int32_t));
    o->randva = (double *)xmalloc((size_t)N * sizeof(double));
    o->randfa = (double *)xmalloc(3 * (size_t)N * sizeof(double));
    o->iseed = in->rand_state;
    /* Nose-Hoover chain start (init_shake tail, src/md.f90:4415-4424) */
    int nc = in->nhchains > 0 ? (in->nhchains < 64 ? in->nhchains : 64) : 0;
    for (int k = 0; k < nc; ++k) { o->qnh[k] = in->nhq; o->vnh[k] = 0; o->xnh[k] = 0; }
    if (nc) o->qnh[0] = in->Ndegf * in->nhq;
    o->d.nhchains = nc;
    /* periodic box (inv_boxl = 1/boxlength, prep_sim) */
    for (int k = 0; k < 3; ++k) {
        o->ibox[k] = in->use_pbc ? 1.0 / in->boxlength[k] : 0.0;
        o->boxc[k] = in->boxcentre[k];
    }
    o->istart_mol = (int32_t *)dupbuf(in->istart_mol, in->use_pbc ? (size_t)in->nmol * sizeof(int32_t) : 0);
    o->d.istart_mol = o->istart_mol;
    return o;
}

void oracle_destroy(void *h) {
    oracle *o = (oracle *)h;
    if (!o) return;
    free(o->x); free(o->v); free(o->xx); free(o->f); free(o->winv); free(o->iwhich); free(o->lrf);
    free(o->pp.a); free(o->pw.a); free(o->ww.a); free(o->qp.a); free(o->qw.a);
    free(o->ex_first); free(o->ex_j); free(o->p14_first); free(o->p14_j);
    free((void *)o->d.rstseq_ij); free((void *)o->d.rstseq_fk); free((void *)o->d.rstseq_flags);
    free((void *)o->d.heavy);
    free((void *)o->d.rstpos_i); free((void *)o->d.rstpos_x); free((void *)o->d.rstdis_i); free((void *)o->d.rstdis_p);
    free((void *)o->d.rstang_i); free((void *)o->d.rstang_p); free((void *)o->d.rstwal_i); free((void *)o->d.rstwal_p);
    free(o->theta_corr); free(o->avtheta); free(o->avn_insh); free(o->n_insh);
    free(o->theta); free(o->tdum); free(o->theta0); free(o->list_sh); free(o->nsort);
    free(o->randva); free(o->randfa);
    free(o);
}

void oracle_set_coords(void *h, const double *x, const double *v) {
    oracle *o = (oracle *)h;
    if (x) memcpy(o->x, x, 3 * (size_t)o->N * sizeof(double));
    if (v) memcpy(o->v, v, 3 * (size_t)o->N * sizeof(double));
}
void oracle_get_coords(void *h, double *x, double *v) {
    oracle *o = (oracle *)h;
    if (x) memcpy(x, o->x, 3 * (size_t)o->N * sizeof(double));
    if (v) memcpy(v, o->v, 3 * (size_t)o->N * sizeof(double));
}

/* ------------------------------------------------------------------ LRF */
/* cgp_centers, src/md.f90:2253-2288 */
/* ----------------------------------------------------------- periodic box */
/* boxlength(k)*nint(d*inv_boxl(k)), the periodic shift of one component as
   every box routine of the reference writes it (Fortran nint rounds halves
   away from zero, as round() does) */
static inline double pbc_shift(const oracle *o, int k, double dk) {
    return o->d.boxlength[k] * round(dk * o->ibox[k]);
}
/* |x_i - x_j|^2, the minimum image in a box (dx = dx - boxlength*nint(dx*inv_boxl),
   r2 = dx**2 + dy**2 + dz**2: nbpplist_box_lrf src/md.f90:8282-8288 and the
   other box list builders); the plain distance in a sphere */
static inline double dist2m(const oracle *o, int i, int j) {
    const double *x = o->x;
    double a = x[3 * i] - x[3 * j], b = x[3 * i + 1] - x[3 * j + 1], c = x[3 * i + 2] - x[3 * j + 2];
    if (o->d.use_pbc) {
        a = a - pbc_shift(o, 0, a);
        b = b - pbc_shift(o, 1, b);
        c = c - pbc_shift(o, 2, c);
    }
    return a * a + b * b + c * c;
}

static void cgp_centers(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int g = 0; g < d->ncgp; ++g) {
        double *r = o->lrf + (size_t)g * NLRF;
        memset(r, 0, NLRF * sizeof(double));
        for (int k = d->cgp_first[g]; k <= d->cgp_last[g]; ++k) {
            int a = d->cgpatom[k];
            r[0] += o->x[3 * a]; r[1] += o->x[3 * a + 1]; r[2] += o->x[3 * a + 2];
        }
        double n = (double)(d->cgp_last[g] - d->cgp_first[g] + 1);
        r[0] /= n; r[1] /= n; r[2] /= n;
    }
}

/* lrf_update(group1, group2), src/md.f90:5896-5981.
   Multipoles of the non-Q atoms of group1 expanded about the centre of group2;
   in a box shifted by the periodic image of group1's switch atom relative to
   that centre (:5905-5917).
   phi2(a,b) and phi3(a,b,c) are stored row-major, index (a*3+b) and (a*9+b*3+c). */
static void lrf_update(oracle *o, int g1, int g2) {
    const qgpu_system_desc *d = &o->d;
    double *r = o->lrf + (size_t)g2 * NLRF;
    double *phi1 = r + 4, *phi2 = r + 7, *phi3 = r + 16;
    double sh[3] = { 0.0, 0.0, 0.0 };
    if (d->use_pbc) {
        const int sw = d->cgp_switch[g1];
        for (int a = 0; a < 3; ++a) sh[a] = pbc_shift(o, a, o->x[3 * sw + a] - r[a]);
    }
    for (int k = d->cgp_first[g1]; k <= d->cgp_last[g1]; ++k) {
        int i = d->cgpatom[k];
        if (is_q(o, i)) continue;
        double dr[3] = { o->x[3 * i] - r[0] - sh[0], o->x[3 * i + 1] - r[1] - sh[1], o->x[3 * i + 2] - r[2] - sh[2] };
        double r2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
        double f0 = d->crg[i] / (r2 * sqrt(r2));
        double f1 = 3.0 * f0 / r2;
        double f2 = -f1 / r2;
        r[3] += f0 * r2;
        for (int a = 0; a < 3; ++a) phi1[a] -= f0 * dr[a];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                phi2[a * 3 + b] += f1 * dr[a] * dr[b] - (a == b ? f0 : 0.0);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c) {
                    double t = (a == b ? dr[c] : 0.0) + (a == c ? dr[b] : 0.0) + (b == c ? dr[a] : 0.0);
                    phi3[a * 9 + b * 3 + c] += f2 * (5.0 * dr[a] * dr[b] * dr[c] - r2 * t);
                }
    }
}

/* lrf_taylor, src/md.f90:5824-5891 */
static void lrf_taylor(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int i = 0; i < o->N; ++i) {
        if (d->excl[i] || is_q(o, i)) continue;
        const double *r = o->lrf + (size_t)o->iwhich[i] * NLRF;
        const double *phi1 = r + 4, *phi2 = r + 7, *phi3 = r + 16;
        double dr[3] = { r[0] - o->x[3 * i], r[1] - o->x[3 * i + 1], r[2] - o->x[3 * i + 2] };
        double V = r[3] + phi1[0] * dr[0] + phi1[1] * dr[1] + phi1[2] * dr[2];
        for (int a = 0; a < 3; ++a)
            V += 0.5 * (phi2[a * 3] * dr[0] + phi2[a * 3 + 1] * dr[1] + phi2[a * 3 + 2] * dr[2]) * dr[a];
        o->E.lrf += 0.5 * d->crg[i] * V;
        for (int a = 0; a < 3; ++a) {
            double df = phi1[a] + phi2[a * 3] * dr[0] + phi2[a * 3 + 1] * dr[1] + phi2[a * 3 + 2] * dr[2];
            for (int b = 0; b < 3; ++b) {
                const double *p = phi3 + a * 9 + b * 3;
                df += 0.5 * (p[0] * dr[0] + p[1] * dr[1] + p[2] * dr[2]) * dr[b];
            }
            o->f[3 * i + a] -= d->crg[i] * df;
        }
    }
}

/* --------------------------------------------------------------- lists */
static inline double dist2(const double *x, int i, int j) {
    double a = x[3 * i] - x[3 * j], b = x[3 * i + 1] - x[3 * j + 1], c = x[3 * i + 2] - x[3 * j + 2];
    return a * a + b * b + c * c;
}
/* count-once parity rule, src/md.f90:8075-8077 (1-based ig+jg has the same
   parity as the 0-based sum) */
static inline int parity_skip(int ig, int jg) {
    return (ig > jg && ((ig + jg) & 1) == 0) || (ig < jg && ((ig + jg) & 1) == 1);
}
static int all_zero(const oracle *o, int i, int j) {
    int ti = o->d.iac[i], tj = o->d.iac[j];
    int c = ljcod(o, ti, tj);
    return (o->d.crg[i] * o->d.crg[j] == 0.0) &&
           (avdw(o, ti, c) * avdw(o, tj, c) == 0.0) &&
           (bvdw(o, ti, c) * bvdw(o, tj, c) == 0.0);
}

/* nbpplist_lrf, src/md.f90:7998-8188 */
static void nbpplist_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcpp * d->Rcpp, rl2 = d->RcLRF * d->RcLRF;
    o->pp.n = 0;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        int is = d->cgp_switch[ig];
        if (d->excl[is]) continue;
        for (int jg = 0; jg < d->ncgp_solute; ++jg) {
            if (parity_skip(ig, jg)) continue;
            int js = d->cgp_switch[jg];
            if (d->excl[js]) continue;
            double r2 = dist2m(o, is, js);
            if (r2 <= rc2) {
                for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka) {
                    int i = d->cgpatom[ka];
                    if (is_q(o, i)) continue;
                    for (int kb = d->cgp_first[jg]; kb <= d->cgp_last[jg]; ++kb) {
                        int j = d->cgpatom[kb];
                        if (ig == jg && i >= j) continue;
                        if (is_q(o, j)) continue;
                        if (all_zero(o, i, j)) continue;
                        if (excluded(o, i, j)) continue;
                        int lj = ljcod(o, d->iac[i], d->iac[j]);
                        if (is14(o, i, j)) lj = 3;
                        nb_push_s(&o->pp, i, j, lj, lj, is, js);
                    }
                }
            } else if (d->use_LRF && r2 <= rl2) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* nbpwlist_lrf, src/md.f90:9300-9429 */
static void nbpwlist_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcpw * d->Rcpw, rl2 = d->RcLRF * d->RcLRF;
    o->pw.n = 0;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        int is = d->cgp_switch[ig];
        if (d->excl[is]) continue;
        for (int jw = 0; jw < d->nwat; ++jw) {
            int ja = d->nat_solute + 3 * jw;
            int jg = o->iwhich[ja];
            if (d->excl[ja]) continue;
            double r2 = dist2m(o, is, ja);
            if (r2 <= rc2) {
                for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka) {
                    int i = d->cgpatom[ka];
                    if (is_q(o, i)) continue;
                    for (int s = 0; s < 3; ++s) {
                        int j = ja + s;
                        if (all_zero(o, i, j)) continue;
                        nb_push_s(&o->pw, i, j, ljcod(o, d->iac[i], d->iac[j]), 0, is, ja);
                    }
                }
            } else if (d->use_LRF && r2 <= rl2) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* Any-atom cut-off of a solute group pair (nbpplis2_lrf, src/md.f90:7518-7545):
   inside when some atom pair of the two groups (Q atoms included) lies within
   the cut-off.  *r2_last is the last distance the reference's loop computed:
   the pair (last atom of ig, last atom of jg) when no pair is inside. */
static int any_atom_inside(const oracle *o, int ig, int jg, double rc2, double *r2_last) {
    const qgpu_system_desc *d = &o->d;
    double r2 = 0.0;
    for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka)
        for (int kb = d->cgp_first[jg]; kb <= d->cgp_last[jg]; ++kb) {
            r2 = dist2(o->x, d->cgpatom[ka], d->cgpatom[kb]);
            if (r2 <= rc2) { *r2_last = r2; return 1; }
        }
    *r2_last = r2;
    return 0;
}

/* nbpplis2_lrf, src/md.f90:7441-7627 (iuse_switch_atom = 0) */
static void nbpplis2_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcpp * d->Rcpp, rl2 = d->RcLRF * d->RcLRF;
    o->pp.n = 0;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        if (d->excl[d->cgp_switch[ig]]) continue;
        for (int jg = 0; jg < d->ncgp_solute; ++jg) {
            if (parity_skip(ig, jg)) continue;
            if (d->excl[d->cgp_switch[jg]]) continue;
            double r2;
            if (any_atom_inside(o, ig, jg, rc2, &r2)) {
                for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka) {
                    int i = d->cgpatom[ka];
                    if (is_q(o, i)) continue;
                    for (int kb = d->cgp_first[jg]; kb <= d->cgp_last[jg]; ++kb) {
                        int j = d->cgpatom[kb];
                        if (is_q(o, j)) continue;
                        if (ig == jg && i >= j) continue;
                        if (excluded(o, i, j)) continue;
                        int lj = ljcod(o, d->iac[i], d->iac[j]);
                        if (is14(o, i, j)) lj = 3;
                        nb_push_s(&o->pp, i, j, lj, lj, -1, -1);
                    }
                }
            } else if (d->use_LRF && r2 <= rl2) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* nbpwlis2_lrf, src/md.f90:8902-9043 (iuse_switch_atom = 0): a solute group
   and a water are inside when some atom of the group lies within Rcpw of the
   water O; otherwise the LRF test uses the group's last atom. */
static void nbpwlis2_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcpw * d->Rcpw, rl2 = d->RcLRF * d->RcLRF;
    o->pw.n = 0;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        if (d->excl[d->cgp_switch[ig]]) continue;
        for (int jw = 0; jw < d->nwat; ++jw) {
            int ja = d->nat_solute + 3 * jw;
            if (d->excl[ja]) continue;
            int jg = o->iwhich[ja];
            int inside = 0;
            double r2 = 0.0;
            for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig] && !inside; ++ka) {
                r2 = dist2(o->x, d->cgpatom[ka], ja);
                if (r2 <= rc2) inside = 1;
            }
            if (inside) {
                for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka) {
                    int i = d->cgpatom[ka];
                    if (is_q(o, i)) continue;
                    for (int s = 0; s < 3; ++s) {
                        int j = ja + s;
                        if (all_zero(o, i, j)) continue;
                        nb_push_s(&o->pw, i, j, ljcod(o, d->iac[i], d->iac[j]), 0, -1, -1);
                    }
                }
            } else if (d->use_LRF && r2 <= rl2) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* nbpplis2_box_lrf, src/md.f90:7241-7439 (periodic box, iuse_switch_atom = 0):
   a solute group pair (count-once parity rule) is inside when some atom pair
   (Q atoms included, ig's atoms outer, jg's inner, minimum images) lies within
   Rcpp; the first such pair is the pair's shift record (nbpp_cgp).  Not
   inside: both LRF updates when some tested pair lies within RcLRF. */
static void nbpplis2_box_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcpp * d->Rcpp, rl2 = d->RcLRF * d->RcLRF;
    o->pp.n = 0;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        for (int jg = 0; jg < d->ncgp_solute; ++jg) {
            if (parity_skip(ig, jg)) continue;
            int inside = 0, inside_lrf = 0, si = -1, sj = -1;
            for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig] && !inside; ++ka)
                for (int kb = d->cgp_first[jg]; kb <= d->cgp_last[jg] && !inside; ++kb) {
                    const int i = d->cgpatom[ka], j = d->cgpatom[kb];
                    const double r2 = dist2m(o, i, j);
                    if (r2 <= rc2) { inside = 1; si = i; sj = j; }
                    else if (r2 <= rl2) inside_lrf = 1;
                }
            if (inside) {
                for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka) {
                    int i = d->cgpatom[ka];
                    if (is_q(o, i)) continue;
                    for (int kb = d->cgp_first[jg]; kb <= d->cgp_last[jg]; ++kb) {
                        int j = d->cgpatom[kb];
                        if (is_q(o, j)) continue;
                        if (ig == jg && i >= j) continue;
                        if (excluded(o, i, j)) continue;
                        int lj = ljcod(o, d->iac[i], d->iac[j]);
                        if (is14(o, i, j)) lj = 3;
                        nb_push_s(&o->pp, i, j, lj, lj, si, sj);
                    }
                }
            } else if (d->use_LRF && inside_lrf) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* nbpwlis2_box_lrf, src/md.f90:8745-8900: a solute group and a water are
   inside when some atom of the group lies within Rcpw of the water O
   (minimum image); that atom and the O are the shift record (nbpw_cgp).  Not
   inside: both LRF updates when some atom of the group lies within RcLRF of
   the O. */
static void nbpwlis2_box_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcpw * d->Rcpw, rl2 = d->RcLRF * d->RcLRF;
    o->pw.n = 0;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        for (int jw = 0; jw < d->nwat; ++jw) {
            const int ja = d->nat_solute + 3 * jw, jg = o->iwhich[ja];
            int inside = 0, inside_lrf = 0, si = -1;
            for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig] && !inside; ++ka) {
                const int i = d->cgpatom[ka];
                const double r2 = dist2m(o, i, ja);
                if (r2 <= rc2) { inside = 1; si = i; }
                else if (r2 <= rl2) inside_lrf = 1;
            }
            if (inside) {
                for (int ka = d->cgp_first[ig]; ka <= d->cgp_last[ig]; ++ka) {
                    int i = d->cgpatom[ka];
                    if (is_q(o, i)) continue;
                    for (int s = 0; s < 3; ++s) {
                        int j = ja + s;
                        if (all_zero(o, i, j)) continue;
                        nb_push_s(&o->pw, i, j, ljcod(o, d->iac[i], d->iac[j]), 0, si, ja);
                    }
                }
            } else if (d->use_LRF && inside_lrf) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* nbqplist, src/md.f90:10215-10322 (built once when Rcq > rexcl_o) */
/* nbqplist_box, src/md.f90:10327-10459: rebuilt at every list update; a
   solute group is inside when one of its atoms lies within Rcq of the Q
   switching atom (minimum image); that atom fixes the group's periodic shift */
static void nbqplist_box(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    o->qp.n = 0;
    if (d->nqat == 0) return;
    double rc2 = d->Rcq * d->Rcq;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        int inside = -1;
        for (int k = d->cgp_first[ig]; k <= d->cgp_last[ig] && inside < 0; ++k)
            if (dist2m(o, d->cgpatom[k], d->qswitch) <= rc2) inside = d->cgpatom[k];
        if (inside < 0) continue;
        for (int k = d->cgp_first[ig]; k <= d->cgp_last[ig]; ++k) {
            int i = d->cgpatom[k];
            if (d->qp_skip[i]) continue;
            for (int iq = 0; iq < d->nqat; ++iq) {
                int lj = ljcod(o, d->iac[i], d->iac[d->iqseq[iq]]);
                for (int p = 0; p < d->nqp14; ++p)
                    if (d->qp14_pairs[2 * p] == iq && d->qp14_pairs[2 * p + 1] == i) lj = 3;
                nb_push_s(&o->qp, iq, i, lj, lj == 2 ? 1 : lj, d->qswitch, inside);
            }
        }
    }
}

/* nbqwlist_box, src/md.f90:10554-10618: waters whose O lies within Rcq of
   the Q switching atom (minimum image), rebuilt at every list update */
static void nbqwlist_box(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    o->qw.n = 0;
    if (d->nqat == 0) return;
    double rc2 = d->Rcq * d->Rcq;
    int ns = d->nat_solute;
    for (int w = 0; w < d->nwat; ++w) {
        int ia = ns + 3 * w;
        if (dist2m(o, ia, d->qswitch) <= rc2)
            for (int iq = 0; iq < d->nqat; ++iq)
                for (int s = 0; s < 3; ++s)
                    nb_push_s(&o->qw, iq, ia + s, ljcod(o, d->iac[ns + s], d->iac[d->iqseq[iq]]), 0, d->qswitch, ia);
    }
}

static void nbqplist(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    if (d->use_pbc) { nbqplist_box(o); return; }
    if (o->qp_done && d->Rcq > d->rexcl_o) return;
    o->qp.n = 0;
    double rc2 = d->Rcq * d->Rcq;
    if (d->nqat == 0) return;
    for (int ig = 0; ig < d->ncgp_solute; ++ig) {
        int ia = d->cgp_switch[ig];
        if (d->excl[ia]) continue;
        int inside = 0;
        if (d->any_atom_lists) {
            /* nbqplis2, src/md.f90:9946-10071: any atom of the group within Rcq */
            for (int k = d->cgp_first[ig]; k <= d->cgp_last[ig] && !inside; ++k) {
                int i = d->cgpatom[k];
                double a = o->x[3 * i] - d->xpcent[0], b = o->x[3 * i + 1] - d->xpcent[1], c = o->x[3 * i + 2] - d->xpcent[2];
                inside = a * a + b * b + c * c <= rc2;
            }
        } else {
            double a = o->x[3 * ia] - d->xpcent[0], b = o->x[3 * ia + 1] - d->xpcent[1], c = o->x[3 * ia + 2] - d->xpcent[2];
            inside = a * a + b * b + c * c <= rc2;
        }
        if (!inside) continue;
        for (int k = d->cgp_first[ig]; k <= d->cgp_last[ig]; ++k) {
            int i = d->cgpatom[k];
            if (d->qp_skip[i]) continue;
            for (int iq = 0; iq < d->nqat; ++iq) {
                int lj = ljcod(o, d->iac[i], d->iac[d->iqseq[iq]]);
                for (int p = 0; p < d->nqp14; ++p)
                    if (d->qp14_pairs[2 * p] == iq && d->qp14_pairs[2 * p + 1] == i) lj = 3;
                int qlj = lj == 2 ? 1 : lj;
                nb_push_s(&o->qp, iq, i, lj, qlj, -1, -1);
            }
        }
    }
    o->qp_done = 1;
}

/* nbwwlist_lrf, src/md.f90:10897-11021 */
static void nbwwlist_lrf(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double rc2 = d->Rcww * d->Rcww, rl2 = d->RcLRF * d->RcLRF;
    o->ww.n = 0;
    int ns = d->nat_solute;
    for (int iw = 0; iw < d->nwat; ++iw) {
        int is = ns + 3 * iw;
        if (d->excl[is]) continue;
        int ig = o->iwhich[is];
        for (int jw = 0; jw < d->nwat; ++jw) {
            int ja = ns + 3 * jw;
            if (d->excl[ja]) continue;
            int jg = o->iwhich[ja];
            if (parity_skip(iw, jw) || iw == jw) continue;
            double r2 = dist2m(o, is, ja);
            if (r2 <= rc2) {
                for (int la = 0; la < 3; ++la)
                    for (int ka = 0; ka < 3; ++ka)
                        nb_push_s(&o->ww, is + la, ja + ka, ljcod(o, d->iac[ns + la], d->iac[ns + ka]), 0, is, ja);
            } else if (d->use_LRF && r2 <= rl2) {
                lrf_update(o, ig, jg);
                lrf_update(o, jg, ig);
            }
        }
    }
}

/* nbqwlist, src/md.f90:10464-10549 (built once when Rcq > rexcl_o) */
static void nbqwlist(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    if (d->use_pbc) { nbqwlist_box(o); return; }
    if (o->qw_done && d->Rcq > d->rexcl_o) return;
    o->qw.n = 0;
    if (d->nqat == 0) return;
    double rc2 = d->Rcq * d->Rcq;
    int ns = d->nat_solute;
    for (int w = 0; w < d->nwat; ++w) {
        int ia = ns + 3 * w;
        if (d->excl[ia]) continue;
        double a = o->x[3 * ia] - d->xpcent[0], b = o->x[3 * ia + 1] - d->xpcent[1], c = o->x[3 * ia + 2] - d->xpcent[2];
        if (a * a + b * b + c * c <= rc2)
            for (int iq = 0; iq < d->nqat; ++iq)
                for (int s = 0; s < 3; ++s)
                    nb_push_s(&o->qw, iq, ia + s, ljcod(o, d->iac[ns + s], d->iac[d->iqseq[iq]]), 0, -1, -1);
    }
    o->qw_done = 1;
}

/* make_pair_lists, LRF branches, src/md.f90:6003-6058: sphere or periodic box,
   switch-atom or any-atom lists (minimum images in the box) */
void oracle_make_pair_lists(void *h) {
    oracle *o = (oracle *)h;
    if (o->d.use_LRF) cgp_centers(o);
    if (o->d.any_atom_lists && o->d.use_pbc) {
        nbpplis2_box_lrf(o);
        nbpwlis2_box_lrf(o);
    } else if (o->d.any_atom_lists) {
        nbpplis2_lrf(o);
        nbpwlis2_lrf(o);
    } else {
        nbpplist_lrf(o);
        nbpwlist_lrf(o);
    }
    nbqplist(o);
    nbwwlist_lrf(o);
    nbqwlist(o);
}

/* list export: which 0 pp, 1 pw, 2 ww, 3 qp, 4 qw; rows (i, j, LJcod) */
int64_t oracle_get_list(void *h, int which, int32_t *out, int64_t cap) {
    oracle *o = (oracle *)h;
    nblist *l = which == 0 ? &o->pp : which == 1 ? &o->pw : which == 2 ? &o->ww : which == 3 ? &o->qp : &o->qw;
    if (out && cap >= l->n)
        for (int64_t k = 0; k < l->n; ++k) {
            out[3 * k] = l->a[k].i; out[3 * k + 1] = l->a[k].j; out[3 * k + 2] = l->a[k].lj;
        }
    return l->n;
}
/* the same records as (i, j, si, sj): si, sj the atom pair whose difference
   fixes the record's periodic shift (-1 in a sphere) */
int64_t oracle_get_list_shift(void *h, int which, int32_t *out, int64_t cap) {
    oracle *o = (oracle *)h;
    nblist *l = which == 0 ? &o->pp : which == 1 ? &o->pw : which == 2 ? &o->ww : which == 3 ? &o->qp : &o->qw;
    if (out && cap >= l->n)
        for (int64_t k = 0; k < l->n; ++k) {
            out[4 * k] = l->a[k].i; out[4 * k + 1] = l->a[k].j;
            out[4 * k + 2] = l->a[k].si; out[4 * k + 3] = l->a[k].sj;
        }
    return l->n;
}
void oracle_get_lrf(void *h, double *out) {
    oracle *o = (oracle *)h;
    memcpy(out, o->lrf, (size_t)o->d.ncgp * NLRF * sizeof(double));
}

/* ---------------------------------------------------------- nonbonds */
#define DX(i, j) double dx1 = o->x[3 * (j)] - o->x[3 * (i)], dx2 = o->x[3 * (j) + 1] - o->x[3 * (i) + 1], \
                        dx3 = o->x[3 * (j) + 2] - o->x[3 * (i) + 2]
/* dx = dx - shift of the record's pair in a box (nonbond_pp_box :13226-13228,
   nonbond_pw_box, nonbond_ww_spc_box :15187-15193, nonbond_qp_box :13989-13991,
   nonbond_qw_spc_box :14627-14633) with shift = boxlength*nint((x[sj]-x[si])*inv_boxl) */
#define BOX_SHIFT(rec) do { if (o->d.use_pbc) { const double *X_ = o->x; \
    const int si_ = (rec).si, sj_ = (rec).sj; \
    dx1 = dx1 - pbc_shift(o, 0, X_[3 * sj_] - X_[3 * si_]); \
    dx2 = dx2 - pbc_shift(o, 1, X_[3 * sj_ + 1] - X_[3 * si_ + 1]); \
    dx3 = dx3 - pbc_shift(o, 2, X_[3 * sj_ + 2] - X_[3 * si_ + 2]); } } while (0)
#define ADD_F(i, j, dv) do { double *F = o->f; \
    F[3*(i)] -= (dv)*dx1; F[3*(i)+1] -= (dv)*dx2; F[3*(i)+2] -= (dv)*dx3; \
    F[3*(j)] += (dv)*dx1; F[3*(j)+1] += (dv)*dx2; F[3*(j)+2] += (dv)*dx3; } while (0)

/* Arithmetic combination rule (ivdw_rule 2; nonbon2_*, src/md.f90:11354-13068):
   aLJ = (a_i + a_j)^6 and bLJ = b_i b_j, V_a = bLJ aLJ^2 / r^12,
   V_b = 2 bLJ aLJ / r^6.  A = bLJ*aLJ*aLJ and B = 2*bLJ*aLJ in the
   reference's association. */
static inline void arith_AB(double ai, double aj, double bi, double bj, double *A, double *B) {
    double a = ai + aj;
    a = a * a;
    a = a * a * a;
    const double b = bi * bj;
    *A = b * a * a;
    *B = 2.0 * b * a;
}

/* nonbond_pp, src/md.f90:13069-13155; arithmetic rule nonbon2_pp :11354-11443 */
static void nonbond_pp(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int64_t k = 0; k < o->pp.n; ++k) {
        int i = o->pp.a[k].i, j = o->pp.a[k].j, c = o->pp.a[k].lj;
        DX(i, j);
        BOX_SHIFT(o->pp.a[k]);
        double r2 = 1.0 / (dx1 * dx1 + dx2 * dx2 + dx3 * dx3), r = sqrt(r2), r6 = r2 * r2 * r2;
        double Vel = d->crg[i] * d->crg[j] * r;
        if (c == 3) Vel *= d->el14_scale;
        double Va, Vb;
        if (d->ivdw_rule == 2) {
            double A, B;
            arith_AB(avdw(o, d->iac[i], c), avdw(o, d->iac[j], c), bvdw(o, d->iac[i], c), bvdw(o, d->iac[j], c), &A, &B);
            Va = A * r6 * r6;
            Vb = B * r6;
        } else {
            Va = r6 * r6 * avdw(o, d->iac[i], c) * avdw(o, d->iac[j], c);
            Vb = r6 * bvdw(o, d->iac[i], c) * bvdw(o, d->iac[j], c);
        }
        double dv = r2 * (-Vel - 12.0 * Va + 6.0 * Vb);
        ADD_F(i, j, dv);
        o->E.pp_el += Vel; o->E.pp_vdw += Va - Vb;
    }
}

/* nonbond_pw, src/md.f90:13282-13365; arithmetic rule nonbon2_pw :11569-11654 */
static void nonbond_pw(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int64_t k = 0; k < o->pw.n; ++k) {
        int i = o->pw.a[k].i, j = o->pw.a[k].j, c = o->pw.a[k].lj;
        double aLJ, bLJ;
        if (d->ivdw_rule == 2)
            arith_AB(avdw(o, d->iac[i], c), avdw(o, d->iac[j], c), bvdw(o, d->iac[i], c), bvdw(o, d->iac[j], c), &aLJ, &bLJ);
        else {
            aLJ = avdw(o, d->iac[i], c) * avdw(o, d->iac[j], c);
            bLJ = bvdw(o, d->iac[i], c) * bvdw(o, d->iac[j], c);
        }
        DX(i, j);
        BOX_SHIFT(o->pw.a[k]);
        double r2 = 1.0 / (dx1 * dx1 + dx2 * dx2 + dx3 * dx3), r = sqrt(r2), r6 = r2 * r2 * r2;
        double Vel = d->crg[i] * d->crg[j] * r, Va = aLJ * (r6 * r6), Vb = bLJ * r6;
        double dv = r2 * (-Vel - 12.0 * Va + 6.0 * Vb);
        ADD_F(i, j, dv);
        o->E.pw_el += Vel; o->E.pw_vdw += Va - Vb;
    }
}

/* nonbond_qp (src/md.f90:13788-13921) and nonbond_qp_qvdw (14097-14230);
   arithmetic rule nonbon2_qp :12221-12376 */
static void nonbond_qp(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    int nt = d->natyps + d->nqat;
    for (int64_t k = 0; k < o->qp.n; ++k) {
        int iq = o->qp.a[k].i, i = d->iqseq[iq], j = o->qp.a[k].j, c = o->qp.a[k].lj, qc = o->qp.a[k].qlj;
        int tj = d->iac[j];
        DX(i, j);
        BOX_SHIFT(o->qp.a[k]);
        double r2 = dx1 * dx1 + dx2 * dx2 + dx3 * dx3;
        if (d->ivdw_rule == 2) {
            const double r6hc = r2 * r2 * r2;
            r2 = 1.0 / r2;
            const double r = sqrt(r2);
            for (int s = 0; s < o->S; ++s) {
                double ai, bi, r6;
                if (!d->qvdw_flag) {
                    ai = avdw(o, d->iac[i], c); bi = bvdw(o, d->iac[i], c);
                    r6 = 1.0 / r6hc;
                } else {
                    int ti = d->qiac[iq * o->S + s], cc = c == 2 ? 1 : c;
                    ai = d->qavdw[ti * 3 + cc - 1]; bi = d->qbvdw[ti * 3 + cc - 1];
                    r6 = 1.0 / (r6hc + d->sc_lookup[((size_t)iq * nt + tj) * o->S + s]);
                }
                double aLJ = ai + avdw(o, tj, c), bLJ = bi * bvdw(o, tj, c);
                aLJ = aLJ * aLJ;
                aLJ = aLJ * aLJ * aLJ;
                double Vel = qcrg(o, iq, s) * d->crg[j] * r;
                if (c == 3) Vel *= d->el14_scale;
                double Va = bLJ * aLJ * aLJ * r6 * r6, Vb = 2.0 * bLJ * aLJ * r6;
                double dv = r2 * (-Vel - (12.0 * Va - 6.0 * Vb) * r6 * r6hc) * d->lambda[s];
                ADD_F(i, j, dv);
                o->EQ[s].qp_el += Vel; o->EQ[s].qp_vdw += Va - Vb;
            }
            continue;
        }
        if (!d->qvdw_flag) {
            r2 = 1.0 / r2;
            double r6 = r2 * r2 * r2, r = sqrt(r2);
            for (int s = 0; s < o->S; ++s) {
                int ti = d->iac[i];
                double aLJ = avdw(o, ti, c) * avdw(o, tj, c), bLJ = bvdw(o, ti, c) * bvdw(o, tj, c);
                double Vel = qcrg(o, iq, s) * d->crg[j] * r;
                if (c == 3) Vel *= d->el14_scale;
                double Va = aLJ * r6 * r6, Vb = bLJ * r6;
                double dv = r2 * (-Vel - 12.0 * Va + 6.0 * Vb) * d->lambda[s];
                ADD_F(i, j, dv);
                o->EQ[s].qp_el += Vel; o->EQ[s].qp_vdw += Va - Vb;
            }
        } else {
            double r6 = r2 * r2 * r2;
            r2 = 1.0 / r2;
            double r = sqrt(r2);
            for (int s = 0; s < o->S; ++s) {
                int ti = d->qiac[iq * o->S + s];
                double aLJ = d->qavdw[ti * 3 + qc - 1] * avdw(o, tj, c);
                double bLJ = d->qbvdw[ti * 3 + qc - 1] * bvdw(o, tj, c);
                double Vel = qcrg(o, iq, s) * d->crg[j] * r;
                if (c == 3) Vel *= d->el14_scale;
                double r6sc = r6 + d->sc_lookup[((size_t)iq * nt + tj) * o->S + s];
                double Va = aLJ / (r6sc * r6sc), Vb = bLJ / r6sc;
                double dv = r2 * (-Vel - (12.0 * Va - 6.0 * Vb) * (r6 / r6sc)) * d->lambda[s];
                ADD_F(i, j, dv);
                o->EQ[s].qp_el += Vel; o->EQ[s].qp_vdw += Va - Vb;
            }
        }
    }
}

/* nonbond_ww_spc, src/md.f90:15021-15119: records walked in strides of 3,
   i cycles through the solvent atoms of the i-water, j is its partner O. */
static void nonbond_ww_spc(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    int ichg = 0;
    for (int64_t k = 0; k < o->ww.n; k += 3) {
        if (ichg > 2) ichg = 0;
        int i = o->ww.a[k].i, j = o->ww.a[k].j;
        double q1 = d->chg_solv[ichg];
        for (int ip = 0; ip < 3; ++ip) {
            int ja = j + ip;
            double q2 = d->chg_solv[ip];
            DX(i, ja);
            BOX_SHIFT(o->ww.a[k]);
            double r2 = dx1 * dx1 + dx2 * dx2 + dx3 * dx3;
            double r6 = r2 * r2 * r2;
            r2 = 1.0 / r2;
            double r = sqrt(r2);
            double Vel = q1 * q2 * r;
            o->E.ww_el += Vel;
            double dv = r2 * (-Vel);
            if (ichg == 0 && ip == 0) {
                int c = ljcod(o, d->iac[i], d->iac[j]);
                double a1 = d->aLJ_solv[0 * 2 + c - 1], a2 = d->aLJ_solv[ip * 2 + c - 1];
                double b1 = d->bLJ_solv[0 * 2 + c - 1], b2 = d->bLJ_solv[ip * 2 + c - 1];
                r6 = 1.0 / r6;
                double Va = a1 * a2 * r6 * r6, Vb = b1 * b2 * r6;
                o->E.ww_vdw += Va - Vb;
                dv += r2 * (-12.0 * Va + 6.0 * Vb);
            }
            ADD_F(i, ja, dv);
        }
        ichg++;
    }
}

/* nonbon2_ww, src/md.f90:12847-12945 (arithmetic rule): Coulomb and LJ on all
   nine atom pairs of a water pair, records walked in strides of 3 as in
   nonbond_ww_spc */
static void nonbon2_ww(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    int ichg = 0;
    for (int64_t k = 0; k < o->ww.n; k += 3) {
        if (ichg > 2) ichg = 0;
        int i = o->ww.a[k].i;
        double q1 = d->chg_solv[ichg];
        for (int ip = 0; ip < 3; ++ip) {
            int ja = o->ww.a[k + ip].j;
            int c = ljcod(o, d->iac[i], d->iac[ja]);
            double aLJ = d->aLJ_solv[ichg * 2 + c - 1] + d->aLJ_solv[ip * 2 + c - 1];
            double bLJ = d->bLJ_solv[ichg * 2 + c - 1] * d->bLJ_solv[ip * 2 + c - 1];
            aLJ = aLJ * aLJ;
            aLJ = aLJ * aLJ * aLJ;
            DX(i, ja);
            BOX_SHIFT(o->ww.a[k]);
            double r2 = 1.0 / (dx1 * dx1 + dx2 * dx2 + dx3 * dx3), r = sqrt(r2), r6 = r2 * r2 * r2, r12 = r6 * r6;
            double Vel = q1 * d->chg_solv[ip] * r;
            double Va = bLJ * aLJ * aLJ * r12, Vb = 2.0 * bLJ * aLJ * r6;
            double dv = r2 * (-Vel - 12.0 * Va + 6.0 * Vb);
            ADD_F(i, ja, dv);
            o->E.ww_el += Vel; o->E.ww_vdw += Va - Vb;
        }
        ichg++;
    }
}

/* nonbon2_qw, src/md.f90:12562-12697 (arithmetic rule): every water atom with
   LJ; softcore by the water atom's type (sc_lookup(iq, iacj, s)) */
static void nonbon2_qw(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    int nt = d->natyps + d->nqat;
    for (int64_t k = 0; k < o->qw.n; k += 3) {
        int iq = o->qw.a[k].i, i = d->iqseq[iq], j0 = o->qw.a[k].j;
        for (int jw = 0; jw < 3; ++jw) {
            int j = j0 + jw, c = o->qw.a[k + jw].lj, tj = d->iac[j];
            double sa = d->aLJ_solv[jw * 2 + c - 1], sb = d->bLJ_solv[jw * 2 + c - 1];
            DX(i, j);
            BOX_SHIFT(o->qw.a[k]);
            double r2 = dx1 * dx1 + dx2 * dx2 + dx3 * dx3;
            const double r6hc = r2 * r2 * r2;
            r2 = 1.0 / r2;
            const double r = sqrt(r2);
            for (int s = 0; s < o->S; ++s) {
                double aLJ, bLJ, r6;
                if (!d->qvdw_flag) {
                    aLJ = avdw(o, d->iac[i], c); bLJ = bvdw(o, d->iac[i], c);
                    r6 = 1.0 / r6hc;
                } else {
                    int ti = d->qiac[iq * o->S + s], cc = c == 2 ? 1 : c;
                    aLJ = d->qavdw[ti * 3 + cc - 1]; bLJ = d->qbvdw[ti * 3 + cc - 1];
                    r6 = 1.0 / (r6hc + d->sc_lookup[((size_t)iq * nt + tj) * o->S + s]);
                }
                aLJ = aLJ + sa;
                bLJ = bLJ * sb;
                aLJ = aLJ * aLJ;
                aLJ = aLJ * aLJ * aLJ;
                double Vel = qcrg(o, iq, s) * d->chg_solv[jw] * r;
                double Va = bLJ * aLJ * aLJ * r6 * r6, Vb = 2.0 * bLJ * aLJ * r6;
                double dv = r2 * (-Vel - (12.0 * Va - 6.0 * Vb) * r6 * r6hc) * d->lambda[s];
                ADD_F(i, j, dv);
                o->EQ[s].qw_el += Vel; o->EQ[s].qw_vdw += Va - Vb;
            }
        }
    }
}

/* nonbond_qw_spc, src/md.f90:14411-14570 */
static void nonbond_qw_spc(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    int nt = d->natyps + d->nqat;
    for (int64_t k = 0; k < o->qw.n; k += 3) {
        int iq = o->qw.a[k].i, i = d->iqseq[iq], j = o->qw.a[k].j, c = o->qw.a[k].lj;
        {
            DX(i, j);
            BOX_SHIFT(o->qw.a[k]);
            double r2 = dx1 * dx1 + dx2 * dx2 + dx3 * dx3;
            double r6hc = r2 * r2 * r2;
            r2 = 1.0 / r2;
            double r = sqrt(r2), r6sc = r6hc, Va = 0, Vb = 0;
            if (!d->qvdw_flag) {
                double r6 = 1.0 / r6hc;
                double aLJ = avdw(o, d->iac[i], c), bLJ = bvdw(o, d->iac[i], c);
                Va = aLJ * d->aLJ_solv[0 * 2 + c - 1] * r6 * r6;
                Vb = bLJ * d->bLJ_solv[0 * 2 + c - 1] * r6;
            }
            double dv = 0;
            for (int s = 0; s < o->S; ++s) {
                if (d->qvdw_flag) {
                    int ti = d->qiac[iq * o->S + s];
                    double aLJ = d->qavdw[ti * 3], bLJ = d->qbvdw[ti * 3];
                    /* softcore indexed by the LJ code (quirk of src/md.f90:14492) */
                    r6sc = r6hc + d->sc_lookup[((size_t)iq * nt + (c - 1)) * o->S + s];
                    Va = aLJ * d->aLJ_solv[0 * 2 + c - 1] / (r6sc * r6sc);
                    Vb = bLJ * d->bLJ_solv[0 * 2 + c - 1] / r6sc;
                }
                double Vel = d->chg_solv[0] * qcrg(o, iq, s) * r;
                dv += r2 * (-Vel - ((12.0 * Va - 6.0 * Vb) * (r6hc / r6sc))) * d->lambda[s];
                o->EQ[s].qw_el += Vel; o->EQ[s].qw_vdw += Va - Vb;
            }
            ADD_F(i, j, dv);
        }
        for (int ip = 1; ip < 3; ++ip) {
            int ja = j + ip;
            DX(i, ja);
            BOX_SHIFT(o->qw.a[k]);
            double r2 = 1.0 / (dx1 * dx1 + dx2 * dx2 + dx3 * dx3), r = sqrt(r2), dv = 0;
            for (int s = 0; s < o->S; ++s) {
                double Vel = d->chg_solv[ip] * qcrg(o, iq, s) * r;
                o->EQ[s].qw_el += Vel;
                dv -= r2 * Vel * d->lambda[s];
            }
            ADD_F(i, ja, dv);
        }
    }
}

/* nonbond_qq, src/md.f90:13491-13636 */
static void nonbond_qq(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    int nt = d->natyps + d->nqat, off = 0;
    for (int s = 0; s < o->S; ++s) {
        for (int k = 0; k < d->nbqq_count[s]; ++k) {
            int p = off + k;
            int iq = d->nbqq_iq[p], i = d->iqseq[iq], j = d->nbqq_j[p], jq = d->nbqq_jq[p], c = d->nbqq_ljcod[p];
            double qi = qcrg(o, iq, s), qj, aLJ, bLJ;
            double els = d->nbqq_elscale[p];
            const int arith = d->ivdw_rule == 2;
            if (arith) {
                /* nonbon2_qq, src/md.f90:11780-11998: sums of the a parameters
                   (a product for the exponential repulsion of a Q-Q pair with code 2) */
                if (!d->qvdw_flag) {
                    int ti = d->iac[i], tj = d->iac[j];
                    aLJ = avdw(o, ti, c) + avdw(o, tj, c);
                    bLJ = bvdw(o, ti, c) * bvdw(o, tj, c);
                    qj = jq >= 0 ? qcrg(o, jq, s) : d->crg[j];
                } else {
                    int ti = d->qiac[iq * o->S + s];
                    aLJ = d->qavdw[ti * 3 + c - 1];
                    bLJ = d->qbvdw[ti * 3 + c - 1];
                    if (jq >= 0) {
                        int tj = d->qiac[jq * o->S + s];
                        qj = qcrg(o, jq, s);
                        if (c == 2) aLJ = aLJ * d->qavdw[tj * 3 + c - 1];
                        else aLJ = aLJ + d->qavdw[tj * 3 + c - 1];
                        bLJ = bLJ * d->qbvdw[tj * 3 + c - 1];
                    } else {
                        if (c == 2) { aLJ = d->qavdw[ti * 3]; bLJ = d->qbvdw[ti * 3]; }
                        int tj = d->iac[j];
                        aLJ = aLJ + avdw(o, tj, c);
                        bLJ = bLJ * bvdw(o, tj, c);
                        qj = d->crg[j];
                    }
                }
            } else if (!d->qvdw_flag) {
                int ti = d->iac[i], tj = d->iac[j];
                aLJ = avdw(o, ti, c) * avdw(o, tj, c);
                bLJ = bvdw(o, ti, c) * bvdw(o, tj, c);
                qj = jq >= 0 ? qcrg(o, jq, s) : d->crg[j];
            } else {
                int ti = d->qiac[iq * o->S + s];
                aLJ = d->qavdw[ti * 3 + c - 1];
                bLJ = d->qbvdw[ti * 3 + c - 1];
                if (jq >= 0) {
                    int tj = d->qiac[jq * o->S + s];
                    aLJ *= d->qavdw[tj * 3 + c - 1];
                    bLJ *= d->qbvdw[tj * 3 + c - 1];
                    qj = qcrg(o, jq, s);
                } else {
                    if (c == 2) { aLJ = d->qavdw[ti * 3]; bLJ = d->qbvdw[ti * 3]; }
                    int tj = d->iac[j];
                    aLJ *= avdw(o, tj, c);
                    bLJ *= bvdw(o, tj, c);
                    qj = d->crg[j];
                }
            }
            DX(i, j);
            double r2 = dx1 * dx1 + dx2 * dx2 + dx3 * dx3;
            double r6hc = r2 * r2 * r2;
            /* softcore column natyps+jq (1-based), natyps for jq = 0: src/md.f90:13561 */
            int col = jq >= 0 ? d->natyps + jq : d->natyps - 1;
            double r6 = r2 * r2 * r2 + d->sc_lookup[((size_t)iq * nt + col) * o->S + s];
            r6 = 1.0 / r6;
            double r12 = r6 * r6;
            r2 = 1.0 / r2;
            double r = sqrt(r2);
            double Vel = qi * qj * r * els, Va, Vb, dv;
            if (c == 3) Vel *= d->el14_scale;
            if (d->qvdw_flag && jq >= 0 && c == 2) {
                Va = aLJ * exp(-bLJ / r);
                Vb = 0.0;
                dv = r2 * (-Vel - bLJ * Va / r) * d->lambda[s];
            } else if (arith) {
                aLJ = aLJ * aLJ;
                aLJ = aLJ * aLJ * aLJ;
                Va = bLJ * aLJ * aLJ * r12;
                Vb = 2.0 * bLJ * aLJ * r6;
                dv = r2 * (-Vel - (12.0 * Va - 6.0 * Vb) * r6 * r6hc) * d->lambda[s];
            } else {
                Va = aLJ * r12;
                Vb = bLJ * r6;
                dv = r2 * (-Vel - (12.0 * Va - 6.0 * Vb) * r6hc * r6) * d->lambda[s];
            }
            ADD_F(i, j, dv);
            if (jq >= 0) { o->EQ[s].qq_el += Vel; o->EQ[s].qq_vdw += Va - Vb; }
            else         { o->EQ[s].qp_el += Vel; o->EQ[s].qp_vdw += Va - Vb; }
        }
        off += d->nbqq_count[s];
    }
}

/* ------------------------------------------------------------ bonded */
static inline const double *X(const oracle *o, int i) { return o->x + 3 * i; }

/* qbond, src/md.f90:17196-17240 (Morse + harmonic) */
static void qbond(oracle *o, int s) {
    const qgpu_system_desc *d = &o->d;
    int w = 2 + o->S;
    for (int b = 0; b < d->nqbond; ++b) {
        int ic = d->qbnd[b * w + 2 + s];
        if (ic <= 0) continue;
        const double *L = d->qbondlib + 4 * (ic - 1);
        int i = d->qbnd[b * w], j = d->qbnd[b * w + 1];
        double rij[3] = { X(o, j)[0] - X(o, i)[0], X(o, j)[1] - X(o, i)[1], X(o, j)[2] - X(o, i)[2] };
        double bl = sqrt(rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
        double db = bl - L[2];
        double fexp = exp(-L[1] * db);
        double be = L[0] * (fexp * fexp - 2.0 * fexp) + 0.5 * L[3] * db * db;
        o->EQ[s].q_bond += be;
        double dv = (2.0 * L[0] * L[1] * (fexp - fexp * fexp) + L[3] * db) * d->lambda[s] / bl;
        for (int a = 0; a < 3; ++a) { o->f[3 * j + a] += rij[a] * dv; o->f[3 * i + a] -= rij[a] * dv; }
        if (b < 256) o->EMorseD[b] = db > 0 ? -(fexp * fexp - 2.0 * fexp) : 1.0;
    }
}

/* shared angle geometry: qangle (src/md.f90:17022-17102), angle (1130-1232) */
static double angle_term(oracle *o, int i, int j, int k, double fk, double ang0, double scale, double *pe) {
    double rji[3], rjk[3];
    for (int a = 0; a < 3; ++a) { rji[a] = X(o, i)[a] - X(o, j)[a]; rjk[a] = X(o, k)[a] - X(o, j)[a]; }
    double bji = sqrt(rji[0] * rji[0] + rji[1] * rji[1] + rji[2] * rji[2]);
    double bjk = sqrt(rjk[0] * rjk[0] + rjk[1] * rjk[1] + rjk[2] * rjk[2]);
    double scp = (rji[0] * rjk[0] + rji[1] * rjk[1] + rji[2] * rjk[2]) / (bji * bjk);
    if (scp > 1.0) scp = 1.0;
    if (scp < -1.0) scp = -1.0;
    double ang = acos(scp), da = ang - ang0;
    *pe = 0.5 * fk * da * da;
    double dv = fk * da * scale;
    double f1 = sin(ang);
    if (fabs(f1) < QREAL_EPS) f1 = QREAL_EPS;
    f1 = -1.0 / f1;
    for (int a = 0; a < 3; ++a) {
        double di = f1 * (rjk[a] / (bji * bjk) - scp * rji[a] / (bji * bji));
        double dk = f1 * (rji[a] / (bji * bjk) - scp * rjk[a] / (bjk * bjk));
        o->f[3 * i + a] += dv * di;
        o->f[3 * k + a] += dv * dk;
        o->f[3 * j + a] -= dv * (di + dk);
    }
    return da;
}

static void qangle(oracle *o, int s) {
    const qgpu_system_desc *d = &o->d;
    int w = 3 + o->S;
    for (int a = 0; a < d->nqangle; ++a) {
        int ic = d->qang[a * w + 3 + s];
        if (ic <= 0) continue;
        const double *L = d->qanglib + 4 * (ic - 1);
        double pe;
        angle_term(o, d->qang[a * w], d->qang[a * w + 1], d->qang[a * w + 2], L[0], L[1], d->lambda[s], &pe);
        o->EQ[s].q_angle += pe;
    }
}

/* torsion geometry shared by qtorsion/qimproper (src/md.f90:17241-17538) and
   torsion/improper/improper2 (17907-18054, 3130-3423).  Returns phi and writes
   the 12 derivative components dp[] of phi w.r.t. the four atoms. */
static double dihedral(const oracle *o, int i, int j, int k, int l, double dp[12]) {
    double rji[3], rjk[3], rkl[3], rnj[3], rnk[3];
    for (int a = 0; a < 3; ++a) {
        rji[a] = X(o, i)[a] - X(o, j)[a];
        rjk[a] = X(o, k)[a] - X(o, j)[a];
        rkl[a] = X(o, l)[a] - X(o, k)[a];
    }
    rnj[0] = rji[1] * rjk[2] - rji[2] * rjk[1];
    rnj[1] = rji[2] * rjk[0] - rji[0] * rjk[2];
    rnj[2] = rji[0] * rjk[1] - rji[1] * rjk[0];
    rnk[0] = -rjk[1] * rkl[2] + rjk[2] * rkl[1];
    rnk[1] = -rjk[2] * rkl[0] + rjk[0] * rkl[2];
    rnk[2] = -rjk[0] * rkl[1] + rjk[1] * rkl[0];
    double bj = sqrt(rnj[0] * rnj[0] + rnj[1] * rnj[1] + rnj[2] * rnj[2]);
    double bk = sqrt(rnk[0] * rnk[0] + rnk[1] * rnk[1] + rnk[2] * rnk[2]);
    double scp = (rnj[0] * rnk[0] + rnj[1] * rnk[1] + rnj[2] * rnk[2]) / (bj * bk);
    if (scp > 1.0) scp = 1.0;
    if (scp < -1.0) scp = -1.0;
    double phi = acos(scp);
    double sgn = rjk[0] * (rnj[1] * rnk[2] - rnj[2] * rnk[1]) + rjk[1] * (rnj[2] * rnk[0] - rnj[0] * rnk[2]) +
                 rjk[2] * (rnj[0] * rnk[1] - rnj[1] * rnk[0]);
    if (sgn < 0) phi = -phi;
    double f1 = sin(phi);
    if (fabs(f1) < QREAL_EPS) f1 = QREAL_EPS;
    f1 = -1.0 / f1;
    double di[3], dl[3], rki[3], rlj[3];
    for (int a = 0; a < 3; ++a) {
        di[a] = f1 * (rnk[a] / (bj * bk) - scp * rnj[a] / (bj * bj));
        dl[a] = f1 * (rnj[a] / (bj * bk) - scp * rnk[a] / (bk * bk));
        rki[a] = rji[a] - rjk[a];
        rlj[a] = -rjk[a] - rkl[a];
    }
    dp[0] = rjk[1] * di[2] - rjk[2] * di[1];
    dp[1] = rjk[2] * di[0] - rjk[0] * di[2];
    dp[2] = rjk[0] * di[1] - rjk[1] * di[0];
    dp[3] = rki[1] * di[2] - rki[2] * di[1] + rkl[1] * dl[2] - rkl[2] * dl[1];
    dp[4] = rki[2] * di[0] - rki[0] * di[2] + rkl[2] * dl[0] - rkl[0] * dl[2];
    dp[5] = rki[0] * di[1] - rki[1] * di[0] + rkl[0] * dl[1] - rkl[1] * dl[0];
    dp[6] = rlj[1] * dl[2] - rlj[2] * dl[1] - rji[1] * di[2] + rji[2] * di[1];
    dp[7] = rlj[2] * dl[0] - rlj[0] * dl[2] - rji[2] * di[0] + rji[0] * di[2];
    dp[8] = rlj[0] * dl[1] - rlj[1] * dl[0] - rji[0] * di[1] + rji[1] * di[0];
    dp[9] = rjk[1] * dl[2] - rjk[2] * dl[1];
    dp[10] = rjk[2] * dl[0] - rjk[0] * dl[2];
    dp[11] = rjk[0] * dl[1] - rjk[1] * dl[0];
    return phi;
}
static void apply_dp(oracle *o, int i, int j, int k, int l, double dv, const double dp[12]) {
    int at[4] = { i, j, k, l };
    for (int n = 0; n < 4; ++n)
        for (int a = 0; a < 3; ++a) o->f[3 * at[n] + a] += dv * dp[3 * n + a];
}

static void qtorsion(oracle *o, int s) {
    const qgpu_system_desc *d = &o->d;
    int w = 4 + o->S;
    for (int p = 0; p < d->nqtor; ++p) {
        int ic = d->qtor[p * w + 4 + s];
        if (ic <= 0) continue;
        const double *L = d->qtorlib + 3 * (ic - 1);
        const int32_t *t = d->qtor + p * w;
        double dp[12];
        double phi = dihedral(o, t[0], t[1], t[2], t[3], dp);
        double arg = L[1] * phi - L[2];
        o->EQ[s].q_torsion += L[0] * (1.0 + cos(arg));
        double dv = -L[1] * L[0] * sin(arg) * d->lambda[s];
        apply_dp(o, t[0], t[1], t[2], t[3], dv, dp);
    }
}

static void qimproper(oracle *o, int s) {
    const qgpu_system_desc *d = &o->d;
    int w = 4 + o->S;
    const double pi = 4.0 * atan(1.0);
    for (int p = 0; p < d->nqimp; ++p) {
        int ic = d->qimp[p * w + 4 + s];
        if (ic <= 0) continue;
        const double *L = d->qimplib + 2 * (ic - 1);
        const int32_t *t = d->qimp + p * w;
        double dp[12];
        double phi = dihedral(o, t[0], t[1], t[2], t[3], dp);
        double arg = phi - L[1];
        arg = arg - 2.0 * pi * nearbyint(arg / (2.0 * pi));
        double dv = L[0] * arg;
        o->EQ[s].q_improper += 0.5 * dv * arg;
        apply_dp(o, t[0], t[1], t[2], t[3], dv * d->lambda[s], dp);
    }
}

/* bond, src/md.f90:1340-1405 */
static double bonds(oracle *o, int b0, int b1) {
    const qgpu_system_desc *d = &o->d;
    double e = 0;
    for (int b = b0; b < b1; ++b) {
        int i = d->bnd[3 * b], j = d->bnd[3 * b + 1], c = d->bnd[3 * b + 2];
        const double *L = d->bondlib + 2 * (c - 1);
        double rij[3] = { X(o, j)[0] - X(o, i)[0], X(o, j)[1] - X(o, i)[1], X(o, j)[2] - X(o, i)[2] };
        double bl = sqrt(rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
        double db = bl - L[1];
        e += 0.5 * L[0] * db * db;
        double dv = L[0] * db / bl;
        for (int a = 0; a < 3; ++a) { o->f[3 * j + a] += rij[a] * dv; o->f[3 * i + a] -= rij[a] * dv; }
    }
    return e;
}
static double angles(oracle *o, int a0, int a1) {
    const qgpu_system_desc *d = &o->d;
    double e = 0;
    for (int a = a0; a < a1; ++a) {
        const int32_t *t = d->ang + 4 * a;
        const double *L = d->anglib + 4 * (t[3] - 1);
        double pe;
        angle_term(o, t[0], t[1], t[2], L[0], L[1], 1.0, &pe);
        e += pe;
    }
    return e;
}
/* torsion, src/md.f90:17907-18054 (loop runs backwards as the reference) */
static double torsions(oracle *o, int p0, int p1) {
    const qgpu_system_desc *d = &o->d;
    double e = 0;
    for (int p = p1 - 1; p >= p0; --p) {
        const int32_t *t = d->tor + 5 * p;
        const float *L = d->torlib + 4 * (t[4] - 1);
        double dp[12];
        double phi = dihedral(o, t[0], t[1], t[2], t[3], dp);
        double arg = (double)L[1] * phi - (double)L[2];
        e += (double)L[0] * (1.0 + cos(arg)) * (double)L[3];
        double dv = -(double)L[1] * (double)L[0] * sin(arg) * (double)L[3];
        apply_dp(o, t[0], t[1], t[2], t[3], dv, dp);
    }
    return e;
}
/* improper (harmonic, src/md.f90:3130-3283) and improper2 (periodic, 3284-3423) */
static double impropers(oracle *o, int p0, int p1) {
    const qgpu_system_desc *d = &o->d;
    const double pi = 4.0 * atan(1.0);
    double e = 0;
    for (int p = p1 - 1; p >= p0; --p) {
        const int32_t *t = d->imp + 5 * p;
        const float *L = d->implib + 2 * (t[4] - 1);
        double dp[12];
        double phi = dihedral(o, t[0], t[1], t[2], t[3], dp);
        double dv;
        if (d->ff_type == 2) {
            double arg = 2.0 * phi - (double)L[1];
            e += (double)L[0] * (1.0 + cos(arg));
            dv = -2.0 * (double)L[0] * sin(arg);
        } else {
            double arg = phi - (double)L[1];
            arg = arg - 2.0 * pi * nearbyint(arg / (2.0 * pi));
            dv = (double)L[0] * arg;
            e += 0.5 * dv * arg;
        }
        apply_dp(o, t[0], t[1], t[2], t[3], dv, dp);
    }
    return e;
}

/* --------------------------------------------------------- restraints */
/* fix_shell, src/md.f90:2816-2864 (no freeze) */
static void fix_shell(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int i = 0; i < d->nat_solute; ++i) {
        if (!(d->excl[i] || d->shell[i])) continue;
        double fk = d->excl[i] ? d->fk_fix : d->fk_pshell;
        double dr[3] = { o->x[3 * i] - d->xtop[3 * i], o->x[3 * i + 1] - d->xtop[3 * i + 1], o->x[3 * i + 2] - d->xtop[3 * i + 2] };
        double e = 0.5 * fk * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        if (d->excl[i]) o->E.rst_fix += e;
        if (d->shell[i]) o->E.rst_shell += e;
        for (int a = 0; a < 3; ++a) o->f[3 * i + a] += fk * dr[a];
    }
}

/* restrain_solvent, src/md.f90:18055-18102 */
static void restrain_solvent(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    double shift = d->fk_wsphere != 0.0 ? sqrt(BOLTZ * o->Tfree / d->fk_wsphere) : 0.0;
    for (int g = d->ncgp_solute; g < d->ncgp; ++g) {
        int i = d->cgp_switch[g];
        if (d->excl[i]) continue;
        double dr[3] = { o->x[3 * i] - d->xwcent[0], o->x[3 * i + 1] - d->xwcent[1], o->x[3 * i + 2] - d->xwcent[2] };
        double b = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        double db = b - (d->rwat - shift), erst, dv;
        if (db > 0) {
            erst = 0.5 * d->fk_wsphere * db * db - d->Dwmz;
            dv = d->fk_wsphere * db / b;
        } else if (b > 0.0) {
            double fexp = exp(d->awmz * db);
            erst = d->Dwmz * (fexp * fexp - 2.0 * fexp);
            dv = -2.0 * d->Dwmz * d->awmz * (fexp - fexp * fexp) / b;
        } else { erst = 0; dv = 0; }
        o->E.rst_solvent_radial += erst;
        for (int a = 0; a < 3; ++a) o->f[3 * i + a] += dv * dr[a];
    }
}

/* p_restrain, sequence restraints, src/md.f90:15484-15576.  An atom takes
   part when heavy, or when the H flag is set and it is not a frozen
   excluded atom (the reference's .and. binds before .or.). */
static void p_restrain_seq(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int ir = 0; ir < d->nrstr_seq; ++ir) {
        const int i0 = d->rstseq_ij[2 * ir], i1 = d->rstseq_ij[2 * ir + 1];
        const double fk = d->rstseq_fk[ir];
        const int ih = d->rstseq_flags[2 * ir], tc = d->rstseq_flags[2 * ir + 1];
#define SEQ_SEL(i) ((d->heavy && d->heavy[i]) || (ih == 1 && !(d->excl[i] && d->excluded_freeze)))
        if (tc == 1 || tc == 2) {
            double dr[3] = { 0, 0, 0 }, w = 0.0;
            for (int i = i0; i <= i1; ++i) {
                if (!SEQ_SEL(i)) continue;
                double m = tc == 2 ? d->mass[d->iac[i]] : 1.0;
                w += m;
                for (int a = 0; a < 3; ++a) dr[a] += (o->x[3 * i + a] - d->xtop[3 * i + a]) * (tc == 2 ? m : 1.0);
            }
            if (w > 0) {
                for (int a = 0; a < 3; ++a) dr[a] /= w;
                double r2 = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
                o->E.rst_protein += 0.5 * fk * r2;
                for (int i = i0; i <= i1; ++i) {
                    if (!SEQ_SEL(i)) continue;
                    double s = tc == 1 ? d->mass[d->iac[i]] / 12.010 : 1.0;
                    for (int a = 0; a < 3; ++a) o->f[3 * i + a] += tc == 1 ? fk * dr[a] * s : fk * dr[a];
                }
            }
        } else {
            for (int i = i0; i <= i1; ++i) {
                if (!SEQ_SEL(i)) continue;
                double dr[3] = { o->x[3 * i] - d->xtop[3 * i], o->x[3 * i + 1] - d->xtop[3 * i + 1],
                                 o->x[3 * i + 2] - d->xtop[3 * i + 2] };
                /* the periodically minimal distance (:15561-15565) */
                if (d->use_pbc)
                    for (int a = 0; a < 3; ++a) dr[a] = dr[a] - pbc_shift(o, a, dr[a]);
                o->E.rst_protein += 0.5 * fk * (dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
                for (int a = 0; a < 3; ++a) o->f[3 * i + a] += fk * dr[a];
            }
        }
#undef SEQ_SEL
    }
}

/* water dipole / radial unit vectors and the angle between them (watpol) */
/* The rest of p_restrain, src/md.f90:15580-15800, in its order: atom position,
   atom-atom distance and angle restraints (state st: 0 = every state, their
   energy added to each state's restraint term; else state st only, force
   weighted by its lambda) and, in a sphere, the half-harmonic wall restraints
   (energy into the protein restraint). */
static void rst_energy(oracle *o, int st, double e) {
    if (st == 0) {
        for (int k = 0; k < o->S; ++k) o->EQ[k].restraint += e;
        if (o->S == 0) o->E.rst_protein += e;
    } else {
        o->EQ[st - 1].restraint += e;
    }
}
static void p_restrain_extra(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    for (int ir = 0; ir < d->nrstr_pos; ++ir) {
        const int i = d->rstpos_i[2 * ir], st = d->rstpos_i[2 * ir + 1];
        const double *p = d->rstpos_x + 6 * ir;
        const double wgt = st ? d->lambda[st - 1] : 1.0;
        double dr[3];
        for (int a = 0; a < 3; ++a) dr[a] = o->x[3 * i + a] - p[a];
        const double e = 0.5 * p[3] * dr[0] * dr[0] + 0.5 * p[4] * dr[1] * dr[1] + 0.5 * p[5] * dr[2] * dr[2];
        for (int a = 0; a < 3; ++a) o->f[3 * i + a] += p[3 + a] * dr[a] * wgt;
        rst_energy(o, st, e);
    }
    for (int ir = 0; ir < d->nrstr_dist; ++ir) {
        const int i = d->rstdis_i[3 * ir], j = d->rstdis_i[3 * ir + 1], st = d->rstdis_i[3 * ir + 2];
        const double d1 = d->rstdis_p[3 * ir], d2 = d->rstdis_p[3 * ir + 1], fk = d->rstdis_p[3 * ir + 2];
        double dr[3];
        for (int a = 0; a < 3; ++a) {
            dr[a] = o->x[3 * j + a] - o->x[3 * i + a];
            if (d->use_pbc) dr[a] = dr[a] - pbc_shift(o, a, dr[a]);
        }
        const double wgt = st ? d->lambda[st - 1] : 1.0;
        const double b = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
        double db;
        if (b < d1) db = b - d1;
        else if (b > d2) db = b - d2;
        else continue;
        const double e = 0.5 * fk * db * db, dv = wgt * fk * db / b;
        for (int a = 0; a < 3; ++a) { o->f[3 * j + a] += dr[a] * dv; o->f[3 * i + a] -= dr[a] * dv; }
        rst_energy(o, st, e);
    }
    for (int ir = 0; ir < d->nrstr_angl; ++ir) {
        const int i = d->rstang_i[4 * ir], j = d->rstang_i[4 * ir + 1], k = d->rstang_i[4 * ir + 2];
        const int st = d->rstang_i[4 * ir + 3];
        const double ang0 = d->rstang_p[2 * ir], fk = d->rstang_p[2 * ir + 1];
        double a1[3], a2[3];
        for (int a = 0; a < 3; ++a) {
            a1[a] = o->x[3 * i + a] - o->x[3 * j + a];
            a2[a] = o->x[3 * k + a] - o->x[3 * j + a];
            if (d->use_pbc) { a1[a] = a1[a] - pbc_shift(o, a, a1[a]); a2[a] = a2[a] - pbc_shift(o, a, a2[a]); }
        }
        const double wgt = st ? d->lambda[st - 1] : 1.0;
        const double r2ij = a1[0] * a1[0] + a1[1] * a1[1] + a1[2] * a1[2];
        const double r2jk = a2[0] * a2[0] + a2[1] * a2[1] + a2[2] * a2[2];
        const double rij = sqrt(r2ij), rjk = sqrt(r2jk);
        double scp = (a1[0] * a2[0] + a1[1] * a2[1] + a1[2] * a2[2]) / (rij * rjk);
        if (scp > 1.0) scp = 1.0;
        if (scp < -1.0) scp = -1.0;
        const double theta = acos(scp);
        const double db = theta - ang0 * (4.0 * atan(1.0) / 180.0);   /* deg2rad, src/md.f90:527-528 */
        const double e = 0.5 * fk * db * db, dv = wgt * fk * db;
        double f1 = sin(theta);
        if (fabs(f1) < QREAL_EPS) f1 = QREAL_EPS;
        f1 = -1.0 / f1;
        double di[3], dk[3];
        for (int a = 0; a < 3; ++a) {
            di[a] = f1 * (a2[a] / (rij * rjk) - scp * a1[a] / r2ij);
            dk[a] = f1 * (a1[a] / (rij * rjk) - scp * a2[a] / r2jk);
        }
        for (int a = 0; a < 3; ++a) {
            o->f[3 * i + a] += dv * di[a];
            o->f[3 * k + a] += dv * dk[a];
            o->f[3 * j + a] -= dv * (di[a] + dk[a]);
        }
        rst_energy(o, st, e);
    }
    if (d->use_pbc) return;
    for (int ir = 0; ir < d->nrstr_wall; ++ir) {
        const int i0 = d->rstwal_i[3 * ir], i1 = d->rstwal_i[3 * ir + 1], ih = d->rstwal_i[3 * ir + 2];
        const double dw = d->rstwal_p[4 * ir], fk = d->rstwal_p[4 * ir + 1];
        const double aM = d->rstwal_p[4 * ir + 2], dM = d->rstwal_p[4 * ir + 3];
        for (int i = i0; i <= i1; ++i) {
            if (!((d->heavy && d->heavy[i]) || ih == 1)) continue;
            double dr[3];
            for (int a = 0; a < 3; ++a) dr[a] = o->x[3 * i + a] - d->xwcent[a];
            const double b = sqrt(dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2]);
            const double db = b - dw;
            double e, dv;
            if (db > 0.0) {
                e = 0.5 * fk * db * db - dM;
                dv = fk * db / b;
            } else {
                const double fexp = exp(aM * db);
                e = dM * (fexp * fexp - 2.0 * fexp);
                dv = -2.0 * dM * aM * (fexp - fexp * fexp) / b;
            }
            o->E.rst_protein += e;
            for (int a = 0; a < 3; ++a) o->f[3 * i + a] += dv * dr[a];
        }
    }
}

static double wat_angle(const oracle *o, int i, double rmu[3], double rcu[3], double *rm, double *rc, double *scp) {
    const double *x = o->x + 3 * i;
    const double *c = o->d.xwcent;
    for (int a = 0; a < 3; ++a) rmu[a] = x[3 + a] + x[6 + a] - 2.0 * x[a];
    *rm = sqrt(rmu[0] * rmu[0] + rmu[1] * rmu[1] + rmu[2] * rmu[2]);
    for (int a = 0; a < 3; ++a) rmu[a] /= *rm;
    for (int a = 0; a < 3; ++a) rcu[a] = x[a] - c[a];
    *rc = sqrt(rcu[0] * rcu[0] + rcu[1] * rcu[1] + rcu[2] * rcu[2]);
    for (int a = 0; a < 3; ++a) rcu[a] /= *rc;
    double s = rmu[0] * rcu[0] + rmu[1] * rcu[1] + rmu[2] * rcu[2];
    if (s > 1.0) s = 1.0;
    if (s < -1.0) s = -1.0;
    *scp = s;
    return acos(s);
}

/* watpol, src/md.f90:18372-18541: radial polarisation restraint of the
   waters in the outer shells.  Shell k is 0-based here (is = k + 1). */
static void watpol(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    const int ns = d->nwpolr_shell, nw = d->nwat, stride = nw + 1;
    const double pi = 4.0 * atan(1.0);
    if (ns <= 0) return;
    for (int k = 0; k < ns; ++k) o->n_insh[k] = 0;
    for (int iw = 0; iw < nw; ++iw) {
        o->theta[iw] = 0; o->theta0[iw] = 0;
        int i = d->nat_solute + 3 * iw;
        if (d->excl[i]) continue;
        double rmu[3], rcu[3], rm, rc, scp;
        o->theta[iw] = wat_angle(o, i, rmu, rcu, &rm, &rc, &scp);
        o->tdum[iw] = o->theta[iw];
        if (rc > d->wshell_rout[ns - 1] - d->wshell_dr[ns - 1]) {
            int is;
            for (is = ns; is >= 2; --is)
                if (rc <= d->wshell_rout[is - 1]) break;
            if (is < 2) is = 1;
            int k = is - 1;
            o->list_sh[k * stride + o->n_insh[k]++] = iw;
        }
    }
    /* selection sort by theta; ties keep the list (water index) order */
    for (int k = 0; k < ns; ++k) {
        int n = o->n_insh[k];
        for (int il = 0; il < n; ++il) {
            double tmin = 2.0 * pi;
            int jmin = -1;
            for (int jl = 0; jl < n; ++jl) {
                int jw = o->list_sh[k * stride + jl];
                if (o->tdum[jw] < tmin) { jmin = jw; tmin = o->theta[jw]; }
            }
            o->nsort[k * stride + il] = jmin;
            if (jmin >= 0) o->tdum[jmin] = 99999.0;
        }
    }
    if (o->istep != 0 && d->itdis_update > 0 && o->istep % d->itdis_update == 0) {
        for (int k = 0; k < ns; ++k) {
            o->avtheta[k] /= (double)d->itdis_update;
            o->avn_insh[k] /= (double)d->itdis_update;
            o->theta_corr[k] = o->theta_corr[k] + o->avtheta[k] - acos(d->wshell_cstb[k]);
            o->avtheta[k] = 0;
            o->avn_insh[k] = 0;
        }
    }
    for (int k = 0; k < ns; ++k) {
        int n = o->n_insh[k];
        if (n == 0) continue;
        double avtdum = 0;
        for (int il = 1; il <= n; ++il) {
            int iw = o->nsort[k * stride + il - 1];
            double arg = 1.0 + (1.0 - 2.0 * (double)il) / (double)n;
            double t0 = acos(arg);
            t0 = t0 - 3.0 * sin(t0) * d->wshell_cstb[k] / 2.0;
            if (t0 < 0) t0 = 0;
            if (t0 > pi) t0 = pi;
            o->theta0[il - 1] = t0;
            avtdum += o->theta[iw];
            double dth = o->theta[iw] - t0 + o->theta_corr[k];
            o->E.rst_water_pol += 0.5 * d->fkwpol * dth * dth;
            double dv = d->fkwpol * dth;
            int i = d->nat_solute + 3 * iw;
            double rmu[3], rcu[3], rm, rc, scp;
            wat_angle(o, i, rmu, rcu, &rm, &rc, &scp);
            double f0 = sin(acos(scp));
            if (fabs(f0) < 1e-14) f0 = 1e-14;
            f0 = -1.0 / f0;
            f0 = dv * f0;
            double f1[3], f2[3];
            for (int a = 0; a < 3; ++a) {
                f1[a] = (rcu[a] - rmu[a] * scp) / rm;
                f2[a] = (rmu[a] - rcu[a] * scp) / rc;
            }
            for (int a = 0; a < 3; ++a) {
                o->f[3 * i + a] += f0 * (-2.0 * f1[a] + f2[a]);
                o->f[3 * i + 3 + a] += f0 * f1[a];
                o->f[3 * i + 6 + a] += f0 * f1[a];
            }
        }
        o->avtheta[k] += avtdum / (double)n;
        o->avn_insh[k] += n;
    }
}

/* offdiag, src/md.f90:15444-15470 */
void oracle_offdiag(void *h, double *Hij_out, double *rkl_out) {
    oracle *o = (oracle *)h;
    const qgpu_system_desc *d = &o->d;
    for (int k = 0; k < d->noffd; ++k) {
        int a = d->iqseq[d->offd_kl[2 * k]], b = d->iqseq[d->offd_kl[2 * k + 1]];
        double r = sqrt(dist2(o->x, b, a));
        double H = d->offd_Amu[2 * k] * exp(-d->offd_Amu[2 * k + 1] * r);
        o->Hij[d->offd_ij[2 * k]][d->offd_ij[2 * k + 1]] = H;
        if (Hij_out) Hij_out[k] = H;
        if (rkl_out) rkl_out[k] = r;
    }
}

/* ------------------------------------------------------- pot_energy */
/* pot_energy, src/md.f90:16015-16221, restricted to `terms` */
void oracle_pot_energy(void *h, int terms, double *d_out, qgpu_energies *E_out, qgpu_qenergy *EQ_out) {
    oracle *o = (oracle *)h;
    const qgpu_system_desc *d = &o->d;
    double kin = o->E.kinetic;
    memset(&o->E, 0, sizeof(o->E));
    o->E.kinetic = kin;
    for (int s = 0; s < o->S; ++s) {
        double lam = o->EQ[s].lambda;
        memset(&o->EQ[s], 0, sizeof(qgpu_qenergy));
        o->EQ[s].lambda = lam;
    }
    memset(o->f, 0, 3 * (size_t)o->N * sizeof(double));
    if (terms & QGPU_TERMS_NONBOND) {
        nonbond_pp(o);
        nonbond_pw(o);
        nonbond_qp(o);
        if (d->natom > d->nat_solute) {
            if (d->ivdw_rule == 2) { nonbon2_ww(o); nonbon2_qw(o); }
            else { nonbond_ww_spc(o); nonbond_qw_spc(o); }
        }
        if (d->use_LRF) lrf_taylor(o);
    }
    if (terms & QGPU_TERMS_BONDED) {
        o->E.p_bond = bonds(o, 0, d->nbonds_solute);
        o->E.w_bond = bonds(o, d->nbonds_solute, d->nbonds);
        o->E.p_angle = angles(o, 0, d->nangles_solute);
        o->E.w_angle = angles(o, d->nangles_solute, d->nangles);
        o->E.p_torsion = torsions(o, 0, d->ntors_solute);
        o->E.w_torsion = torsions(o, d->ntors_solute, d->ntors);
        o->E.p_improper = impropers(o, 0, d->nimps_solute);
        o->E.w_improper = impropers(o, d->nimps_solute, d->nimps);
    }
    if (terms & QGPU_TERMS_RESTRAINT) {
        /* pot_energy order, src/md.f90:16113-16125; no sphere restraints in a box */
        if (!d->use_pbc) fix_shell(o);
        p_restrain_seq(o);
        p_restrain_extra(o);
        if (d->nwat > 0 && !d->use_pbc) {
            restrain_solvent(o);
            if (d->wpol_restr) watpol(o);
        }
    }
    if (terms & QGPU_TERMS_QQ) nonbond_qq(o);
    if (terms & QGPU_TERMS_QBONDED)
        for (int s = 0; s < o->S; ++s) { qbond(o, s); qangle(o, s); qtorsion(o, s); qimproper(o, s); }
    for (int s = 0; s < o->S; ++s) {
        qgpu_qenergy *q = &o->EQ[s];
        q->qx_el = q->qq_el + q->qp_el + q->qw_el;
        q->qx_vdw = q->qq_vdw + q->qp_vdw + q->qw_vdw;
        q->total = q->q_bond + q->q_angle + q->q_torsion + q->q_improper + q->qx_el + q->qx_vdw + q->restraint;
        o->E.q_bond += q->q_bond * q->lambda;
        o->E.q_angle += q->q_angle * q->lambda;
        o->E.q_torsion += q->q_torsion * q->lambda;
        o->E.q_improper += q->q_improper * q->lambda;
        o->E.qx_el += q->qx_el * q->lambda;
        o->E.qx_vdw += q->qx_vdw * q->lambda;
        o->E.rst_protein += q->restraint * q->lambda;
    }
    qgpu_energies *e = &o->E;
    e->rst_total = e->rst_fix + e->rst_shell + e->rst_protein + e->rst_solvent_radial + e->rst_water_pol;
    e->potential = e->p_bond + e->w_bond + e->p_angle + e->w_angle + e->p_torsion + e->p_improper + e->pp_el +
                   e->pp_vdw + e->pw_el + e->pw_vdw + e->ww_el + e->ww_vdw + e->q_bond + e->q_angle +
                   e->q_torsion + e->q_improper + e->qx_el + e->qx_vdw + e->rst_total + e->lrf;
    if (d_out) memcpy(d_out, o->f, 3 * (size_t)o->N * sizeof(double));
    if (E_out) *E_out = o->E;
    if (EQ_out) memcpy(EQ_out, o->EQ, (size_t)o->S * sizeof(qgpu_qenergy));
}

/* ------------------------------------------------------------- SHAKE */
/* shake, src/md.f90:17581-17679.  Returns average iterations per molecule
   (the reference divides by nmol), or -1 when a molecule fails to converge. */
int oracle_shake_arrays(void *h, const double *xx, double *x) {
    oracle *o = (oracle *)h;
    const qgpu_system_desc *d = &o->d;
    int total = 0;
    uint8_t ready[64];
    for (int m = 0; m < d->shake_molecules; ++m) {
        int c0 = d->shake_first[m], nc = d->shake_first[m + 1] - c0;
        if (nc > 64) return -2;
        memset(ready, 0, sizeof(ready));
        int nits = 0;
        for (;;) {
            for (int c = 0; c < nc; ++c) {
                if (ready[c]) continue;
                int i = d->shake_i[c0 + c], j = d->shake_j[c0 + c];
                double d2 = d->shake_dist2[c0 + c];
                double xij[3], xxij[3];
                for (int a = 0; a < 3; ++a) { xij[a] = x[3 * i + a] - x[3 * j + a]; xxij[a] = xx[3 * i + a] - xx[3 * j + a]; }
                double xij2 = xij[0] * xij[0] + xij[1] * xij[1] + xij[2] * xij[2];
                double diff = d2 - xij2;
                if (fabs(diff) < SHAKE_TOL * d2) ready[c] = 1;
                double scp = xij[0] * xxij[0] + xij[1] * xxij[1] + xij[2] * xxij[2];
                double corr = diff / (2.0 * scp * (o->winv[i] + o->winv[j]));
                for (int a = 0; a < 3; ++a) {
                    x[3 * i + a] += xxij[a] * corr * o->winv[i];
                    x[3 * j + a] -= xxij[a] * corr * o->winv[j];
                }
            }
            nits++;
            int all = 1;
            for (int c = 0; c < nc; ++c) all &= ready[c];
            if (all) break;
            if (nits >= SHAKE_MAX_ITER) return -1;
        }
        total += nits;
    }
    return d->shake_molecules ? total / (d->shake_molecules) : 0;
}

/* ------------------------------------------------------ thermostat/MD */
/* randm, src/md.f90:17543-17577 (multiplicative congruential generator) */
static double randm(oracle *o, int32_t *ig) {
    const int32_t m = 100000000, m1 = 10000, mult = 31415821;
    if (!o->rand_new) { o->rand_new = 1; o->irand = abs(*ig) % m; }
    int32_t ih = o->irand / m1, il = o->irand % m1, mh = mult / m1, ml = mult % m1;
    o->irand = ((ih * ml + il * mh) % m1) * m1 + il * ml;
    o->irand = (o->irand + 1) % m;
    double r = (double)(o->irand / 10) * 10 / (double)m;
    if (r <= 0.0 || r > 1.0) r = 0.0;
    *ig = o->irand;
    return r;
}
/* gauss, src/md.f90:2866-2882 */
static double gauss(oracle *o, double am, double sd, int32_t *ig) {
    double a = 0;
    for (int i = 0; i < 12; ++i) a += randm(o, ig);
    return (a - 6.0) * sd + am;
}
/* maxwell, src/md.f90:6075-6094 */
void oracle_maxwell(void *h, double Tmaxw, int32_t seed) {
    oracle *o = (oracle *)h;
    double kT = BOLTZ * Tmaxw;
    for (int i = 0; i < o->N; ++i) {
        double sd = sqrt(kT / o->d.mass[o->d.iac[i]]);
        for (int a = 0; a < 3; ++a) o->v[3 * i + a] = gauss(o, 0.0, sd, &seed);
    }
}
/* initial_shaking, src/md.f90:4430-4450 */
int oracle_initial_shaking(void *h) {
    oracle *o = (oracle *)h;
    size_t n3 = 3 * (size_t)o->N;
    memcpy(o->xx, o->x, n3 * sizeof(double));
    int r1 = oracle_shake_arrays(o, o->xx, o->x);
    if (r1 < 0) return r1;
    for (size_t k = 0; k < n3; ++k) o->xx[k] = o->x[k] - o->d.dt * o->v[k];
    int r2 = oracle_shake_arrays(o, o->x, o->xx);
    if (r2 < 0) return r2;
    for (size_t k = 0; k < n3; ++k) o->v[k] = (o->x[k] - o->xx[k]) / o->d.dt;
    return 0;
}
/* stop_cm_translation, src/md.f90:17784-17816 */
void oracle_stop_cm_translation(void *h) {
    oracle *o = (oracle *)h;
    double tot = 0, vcm[3] = { 0, 0, 0 };
    for (int i = 0; i < o->N; ++i) {
        double m = o->d.mass[o->d.iac[i]];
        tot += m;
        for (int a = 0; a < 3; ++a) vcm[a] += m * o->v[3 * i + a];
    }
    for (int a = 0; a < 3; ++a) vcm[a] /= tot;
    for (int i = 0; i < o->N; ++i)
        for (int a = 0; a < 3; ++a) o->v[3 * i + a] -= vcm[a];
}

/* temperature, src/md.f90:6098-6190 (Berendsen scale factors) */
void oracle_temperature(void *h, double *out4) {
    oracle *o = (oracle *)h;
    const qgpu_system_desc *d = &o->d;
    double Tsu = 0, Tfsu = 0, Tsv = 0, Tfsv = 0;
    for (int i = 0; i < o->N; ++i) {
        const double *v = o->v + 3 * i;
        double ek = 0.5 * d->mass[d->iac[i]] * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (i < d->nat_solute) { Tsu += ek; if (!d->excl[i]) Tfsu += ek; }
        else { Tsv += ek; if (!d->excl[i]) Tfsv += ek; }
    }
    double Tfree = Tfsv + Tfsu, Temp = Tsu + Tsv;
    o->E.kinetic = Temp;
    Temp = 2.0 * Temp / BOLTZ / (double)d->Ndegf;
    Tfree = 2.0 * Tfree / BOLTZ / (double)d->Ndegfree;
    if (d->detail_temps) {
        Tfsu = 2.0 * Tfsu / BOLTZ / (double)d->Ndegfree_solute;
        Tfsv = 2.0 * Tfsv / BOLTZ / (double)d->Ndegfree_solvent;
    }
    double ts = o->Tscale_solvent, tu = o->Tscale_solute;
    if (d->thermostat != 0) {
        /* only the Berendsen thermostat scales (src/md.f90:6166) */
    } else if (d->separate_scaling) {
        if (Tfsv != 0) ts = d->Temp0 / Tfsv - 1.0;
        ts = sqrt(1 + d->dt / d->tau_T * ts);
        if (Tfsu != 0) tu = d->Temp0 / Tfsu - 1.0;
        tu = sqrt(1 + d->dt / d->tau_T * tu);
    } else {
        if (Tfree != 0) ts = d->Temp0 / Tfree - 1.0;
        ts = sqrt(1 + d->dt / d->tau_T * ts);
        tu = ts;
    }
    o->Temp = Temp; o->Tfree = Tfree; o->Tfree_solute = Tfsu; o->Tfree_solvent = Tfsv;
    o->Tscale_solute = tu; o->Tscale_solvent = ts;
    if (out4) { out4[0] = Temp; out4[1] = Tfree; out4[2] = tu; out4[3] = ts; }
}

/* newvel_ber, src/md.f90:6194-6223; with velocity-verlet the velocity update
   is applied a second time after the position update */
static void newvel_ber(oracle *o, double step, double ts, int a0, int a1) {
    const double dt = o->d.dt;
    const int vv = o->d.integrator == 1;
    for (int i = a0; i < a1; ++i)
        for (int a = 0; a < 3; ++a) {
            int k = 3 * i + a;
            o->v[k] = (o->v[k] - o->f[k] * o->winv[i] * step) * ts;
            o->xx[k] = o->x[k];
            o->x[k] = o->x[k] + o->v[k] * dt;
            if (vv) o->v[k] = (o->v[k] - o->f[k] * o->winv[i] * step) * ts;
        }
}

/* newvel_lan, src/md.f90:6225-6270: random forces for every atom first
   (uniform: randva*(r - 1/2); Gaussian: gauss(0, randva)), then the update */
static void newvel_lan(oracle *o, double step, double lfriction) {
    const double dt = o->d.dt;
    const int vv = o->d.integrator == 1;
    for (int i = 0; i < o->N; ++i)
        for (int a = 0; a < 3; ++a)
            o->randfa[3 * i + a] = o->d.langevin_gauss ? gauss(o, 0.0, o->randva[i], &o->iseed)
                                                       : o->randva[i] * (randm(o, &o->iseed) - 0.5);
    for (int i = 0; i < o->N; ++i)
        for (int a = 0; a < 3; ++a) {
            int k = 3 * i + a;
            o->v[k] = (o->v[k] * lfriction) - (o->f[k] - o->randfa[k]) * o->winv[i] * step;
            o->xx[k] = o->x[k];
            o->x[k] = o->x[k] + o->v[k] * dt;
            if (vv) o->v[k] = (o->v[k] * lfriction) - (o->f[k] - o->randfa[k]) * o->winv[i] * step;
        }
}

/* newvel_nos, src/md.f90:6272-6298 */
static void newvel_nos(oracle *o, double step) {
    const double dt = o->d.dt;
    const int vv = o->d.integrator == 1;
    for (int i = 0; i < o->N; ++i)
        for (int a = 0; a < 3; ++a) {
            int k = 3 * i + a;
            o->v[k] = o->v[k] - o->f[k] * o->winv[i] * step;
            o->xx[k] = o->x[k];
            o->x[k] = o->x[k] + o->v[k] * dt;
            if (vv) o->v[k] = o->v[k] - o->f[k] * o->winv[i] * step;
        }
}

/* nh_prop, src/md.f90:6300-6345 (chain index k = i - 1) */
static void nh_prop(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    const int nc = d->nhchains;
    if (nc < 1) return;
    const double dt2 = 0.5 * d->dt, dt4 = 0.5 * dt2, dt8 = 0.5 * dt4;
    const double kbT = BOLTZ * d->Temp0;
    double expf = 1.0, sc;
    o->Gnh[0] = d->Ndegf * BOLTZ * (o->Temp - d->Temp0) / o->qnh[0];
    for (int i = 1; i < nc; ++i) o->Gnh[i] = (o->qnh[i - 1] * o->vnh[i - 1] * o->vnh[i - 1] - kbT) / o->qnh[i];
    o->vnh[nc - 1] = o->vnh[nc - 1] + o->Gnh[nc - 1] * dt4;
    o->xnh[nc - 1] = o->xnh[nc - 1] + o->vnh[nc - 1] * dt2;
    for (int i = nc - 2; i >= 0; --i) {
        expf = exp(-dt8 * o->vnh[i + 1]);
        o->vnh[i] = (o->vnh[i] * expf + o->Gnh[i] * dt4) * expf;
        o->xnh[i] = o->xnh[i] + o->vnh[i] * dt2;
    }
    sc = exp(-o->vnh[0] * dt2);
    for (size_t k = 0; k < 3 * (size_t)o->N; ++k) o->v[k] = o->v[k] * sc;
    o->Gnh[0] = d->Ndegf * BOLTZ * (sc * sc * o->Temp - d->Temp0) / o->qnh[0];
    o->vnh[0] = (o->vnh[0] * expf + o->Gnh[0] * dt4) * expf;
    for (int i = 1; i < nc - 1; ++i) {
        expf = exp(-dt8 * o->vnh[i + 1]);
        o->Gnh[i] = (o->qnh[i - 1] * o->vnh[i - 1] * o->vnh[i - 1] - kbT) / o->qnh[i];
        o->vnh[i] = (o->vnh[i] * expf + o->Gnh[i] * dt4) * expf;
    }
    if (nc > 1) {
        o->Gnh[nc - 1] = (o->qnh[nc - 2] * o->vnh[nc - 2] * o->vnh[nc - 2] - kbT) / o->qnh[nc - 1];
        o->vnh[nc - 1] = o->vnh[nc - 1] + o->Gnh[nc - 1] * dt4;
    }
}

/* put_back_in_box, src/md.f90:18740-18857: the box centre follows the mean
   solute position unless rigid_box_centre; every molecule of the selected
   kind whose mass centre lies outside the box moves by one box length per
   axis. */
static void put_back_in_box(oracle *o) {
    const qgpu_system_desc *d = &o->d;
    if (!d->rigid_box_centre) {
        const int n = d->nat_solute > 0 ? d->nat_solute : d->natom;
        double c[3] = { 0.0, 0.0, 0.0 };
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) c[a] += o->x[3 * i + a];
        for (int a = 0; a < 3; ++a) o->boxc[a] = c[a] / n;
    }
    double hi[3], lo[3];
    for (int a = 0; a < 3; ++a) {
        hi[a] = o->boxc[a] + d->boxlength[a] / 2;
        lo[a] = o->boxc[a] - d->boxlength[a] / 2;
    }
    const int m0 = d->put_solute_back ? 0 : d->nsolute_mol;
    const int m1 = d->put_solvent_back ? d->nmol : d->nsolute_mol;
    for (int m = m0; m < m1; ++m) {
        const int a0 = o->istart_mol[m], a1 = m + 1 < d->nmol ? o->istart_mol[m + 1] : d->natom;
        double cm[3] = { 0.0, 0.0, 0.0 }, mt = 0.0;
        for (int j = a0; j < a1; ++j) mt += d->mass[d->iac[j]];
        for (int j = a0; j < a1; ++j)
            for (int a = 0; a < 3; ++a) cm[a] += o->x[3 * j + a] * d->mass[d->iac[j]];
        for (int a = 0; a < 3; ++a) {
            cm[a] = cm[a] * (1.0 / mt);
            double mv = cm[a] > hi[a] ? -d->boxlength[a] : (cm[a] < lo[a] ? d->boxlength[a] : 0.0);
            if (mv != 0.0)
                for (int j = a0; j < a1; ++j) o->x[3 * j + a] = o->x[3 * j + a] + mv;
        }
    }
}
void oracle_put_back_in_box(void *h) { put_back_in_box((oracle *)h); }

/* md_run, src/md.f90:6440-6664: thermostat constants before the loop, then
   per step lists (every NBcycle steps), pot_energy, offdiag, the thermostat's
   velocity/position update, SHAKE (+ a second nh_prop), temperature.  The step
   counter continues across calls.  Energies of every step are written to
   E_rows[nsteps] / EQ_rows[nsteps*nstates] when given.  Returns 0 or a
   QGPU_E_* status. */
int oracle_md_run(void *h, int32_t nsteps, int32_t terms, qgpu_energies *E_rows, qgpu_qenergy *EQ_rows,
                  double *temps) {
    oracle *o = (oracle *)h;
    const qgpu_system_desc *d = &o->d;
    size_t n3 = 3 * (size_t)o->N;
    const double dv_mod = d->integrator == 1 ? 0.5 * d->dt : d->dt;
    double dv_friction = 1.0;
    if (d->thermostat == 1) {
        dv_friction = 1.0 - d->friction * dv_mod;
        double gkT = (d->langevin_gauss ? 2.0 : 24.0) * d->friction * BOLTZ * d->Temp0 / dv_mod;
        for (int i = 0; i < o->N; ++i) o->randva[i] = sqrt(gkT / o->winv[i]);
    }
    for (int step = 0; step < nsteps; ++step, ++o->istep) {
        if (o->istep % d->NBcycle == 0) {
            if (d->use_pbc && (d->put_solute_back || d->put_solvent_back)) put_back_in_box(o);
            oracle_make_pair_lists(o);
        }
        oracle_pot_energy(o, terms, NULL, NULL, NULL);
        if (d->noffd > 0) oracle_offdiag(o, NULL, NULL);
        if (d->thermostat == 1) {
            newvel_lan(o, dv_mod, dv_friction);
        } else if (d->thermostat == 2) {
            nh_prop(o);
            newvel_nos(o, dv_mod);
        } else {
            newvel_ber(o, dv_mod, o->Tscale_solute, 0, d->nat_solute);
            newvel_ber(o, dv_mod, o->Tscale_solvent, d->nat_solute, d->natom);
        }
        if (d->shake_molecules > 0) {
            if (oracle_shake_arrays(o, o->xx, o->x) < 0) return QGPU_E_SHAKE;
            for (size_t k = 0; k < n3; ++k) o->v[k] = (o->x[k] - o->xx[k]) / d->dt;
            if (d->thermostat == 2) nh_prop(o);
        }
        oracle_temperature(o, NULL);
        if (o->Temp != o->Temp) return QGPU_E_NAN;
        if (E_rows) E_rows[step] = o->E;
        if (EQ_rows) memcpy(EQ_rows + (size_t)step * o->S, o->EQ, (size_t)o->S * sizeof(qgpu_qenergy));
        if (temps) temps[step] = o->Temp;
    }
    return 0;
}

/* The energies after the MD loop (src/md.f90:6687-6693): lists and
   pot_energy at the final coordinates, with the step counter at nsteps. */
void oracle_final_energy(void *h, int terms, qgpu_energies *E, qgpu_qenergy *EQ) {
    oracle *o = (oracle *)h;
    oracle_make_pair_lists(o);
    oracle_pot_energy(o, terms, NULL, E, EQ);
}

/* -------------------------------------------------------- inspection */
void oracle_get_energies(void *h, qgpu_energies *E, qgpu_qenergy *EQ) {
    oracle *o = (oracle *)h;
    if (E) *E = o->E;
    if (EQ) memcpy(EQ, o->EQ, (size_t)o->S * sizeof(qgpu_qenergy));
}
/* the randm state the next random number continues from (the reference's
   iseed after its last randm call) */
int32_t oracle_rand_state(void *h) {
    oracle *o = (oracle *)h;
    return o->rand_new ? o->irand : abs(o->iseed) % 100000000;
}
int oracle_sizeof_desc(void) { return (int)sizeof(qgpu_system_desc); }
int oracle_sizeof_energies(void) { return (int)sizeof(qgpu_energies); }
int oracle_sizeof_qenergy(void) { return (int)sizeof(qgpu_qenergy); }

/* ------------------------------------------------------------- qfep */
/* One Fortran unformatted sequential record (4-byte length markers before
   and after the payload).  Returns the payload length, -1 at end of file,
   -2 on a malformed record; the payload is copied when it fits in cap. */
static long read_record(FILE *f, unsigned char *buf, long cap) {
    int32_t n, m;
    if (fread(&n, 4, 1, f) != 1) return -1;
    if (n < 0) return -2;
    if (n <= cap) {
        if (n && fread(buf, 1, (size_t)n, f) != (size_t)n) return -2;
    } else if (fseek(f, n, SEEK_CUR) != 0) return -2;
    if (fread(&m, 4, 1, f) != 1 || m != n) return -2;
    return n;
}

/* qfep Part 1 (src/qfep.f90:247-661) on nfiles energy files in lambda order:
   reads each file's header (canary 1337) and frames (get_ene, src/nrgy.f90:
   147-188: nstates state records, then the OFFD record), takes lambda of the
   window from the state records, V = EQ(s)%total, skips nskip points, and
   forms dgf / dgr / dG exactly as qfep.  npts[nfiles] gets the frame counts.
   Returns 0, or -1 when a file cannot be read. */
int oracle_qfep_fep(int nfiles, const char **paths, int nstates, double rt, int nskip, double *dgf_out,
                    double *dgr_out, double *dg_out, int *npts) {
    if (nfiles < 1 || nstates < 1 || nstates > QGPU_MAX_STATES) return -1;
    double **V = (double **)xmalloc((size_t)nfiles * sizeof(double *));
    double *lam = (double *)xmalloc((size_t)nfiles * nstates * sizeof(double));
    int rc = 0;
    unsigned char buf[4096];
    for (int fi = 0; fi < nfiles && !rc; ++fi) {
        FILE *f = fopen(paths[fi], "rb");
        if (!f) { rc = -1; break; }
        long n = read_record(f, buf, sizeof buf);
        int32_t canary = 0;
        if (n >= 4) memcpy(&canary, buf, 4);
        if (n < 4 || canary != 1337) { fclose(f); rc = -1; break; }
        size_t cap = 64, np = 0;
        V[fi] = (double *)xmalloc(cap * nstates * sizeof(double));
        for (;;) {
            double row[QGPU_MAX_STATES];
            int s;
            for (s = 0; s < nstates; ++s) {
                n = read_record(f, buf, sizeof buf);
                if (n < 4 + 8 * 15) break;
                double lm, tot;
                memcpy(&lm, buf + 4, 8);
                memcpy(&tot, buf + 12, 8);
                if (np == 0) lam[(size_t)fi * nstates + s] = lm;
                row[s] = tot;
            }
            if (s < nstates) break;
            if (read_record(f, buf, sizeof buf) < 0) break;   /* OFFD */
            if (np == cap) { cap *= 2; V[fi] = (double *)realloc(V[fi], cap * nstates * sizeof(double)); }
            memcpy(V[fi] + np * nstates, row, (size_t)nstates * sizeof(double));
            ++np;
        }
        fclose(f);
        npts[fi] = (int)np;
    }
    if (!rc) {
        double *dgf = (double *)xmalloc((size_t)(nfiles + 2) * sizeof(double));
        double *dgr = (double *)xmalloc((size_t)(nfiles + 2) * sizeof(double));
        for (int fi = 0; fi + 1 < nfiles; ++fi) {
            double sum = 0.0;
            for (int p = nskip; p < npts[fi]; ++p) {
                double v1 = 0.0, v2 = 0.0;
                for (int s = 0; s < nstates; ++s) {
                    v1 += lam[(size_t)fi * nstates + s] * V[fi][(size_t)p * nstates + s];
                    v2 += lam[(size_t)(fi + 1) * nstates + s] * V[fi][(size_t)p * nstates + s];
                }
                sum += exp(-(v2 - v1) / rt);
            }
            sum /= (double)(npts[fi] - nskip);
            dgf[fi] = -rt * log(sum);
        }
        for (int fi = nfiles - 1; fi >= 1; --fi) {
            double sum = 0.0;
            for (int p = nskip; p < npts[fi]; ++p) {
                double v1 = 0.0, v2 = 0.0;
                for (int s = 0; s < nstates; ++s) {
                    v1 += lam[(size_t)fi * nstates + s] * V[fi][(size_t)p * nstates + s];
                    v2 += lam[(size_t)(fi - 1) * nstates + s] * V[fi][(size_t)p * nstates + s];
                }
                sum += exp(-(v2 - v1) / rt);
            }
            sum /= (double)(npts[fi] - nskip);
            dgr[fi] = -rt * log(sum);
        }
        double g = 0.0;
        for (int fi = 0; fi < nfiles; ++fi) {
            if (fi > 0) g = g + 0.5 * (dgf[fi - 1] - dgr[fi]);
            if (dg_out) dg_out[fi] = g;
            if (dgf_out) dgf_out[fi] = fi + 1 < nfiles ? dgf[fi] : 0.0;
            if (dgr_out) dgr_out[fi] = fi > 0 ? dgr[fi] : 0.0;
        }
        free(dgf); free(dgr);
    }
    for (int fi = 0; fi < nfiles; ++fi) free(V[fi]);
    free(V); free(lam);
    return rc;
}

/* ------------------------------------------------------------------------
 * make_qconn (src/md.f90:9582-9620), find_bonded (:9625-9680), nbqqlist
 * (:9716-9804) and the Q-atom / solute skip data that nbqplist reads
 * (:10288 any(qconn(:,j,:) <= 3), :10306 qconn(1,j,iq) == 4 -> LJcod 3),
 * restated from the topology.  Indices are 0-based; the Fortran 1-based
 * levels are kept (1 = the Q atom itself, 2 bonded, 3 angle, 4 torsion,
 * 9 = farther, 0 = special exclusion).
 *
 * Inputs: nsol solute atoms, nq Q atoms in ns states; iqseq[nq]; iqatom[nsol]
 * (-1 = not a Q atom); iac[nsol] and the natyps x natyps ljcod matrix;
 * the solute bond list before shrink_topology (nb rows of i, j, cod; cod 0 =
 * redefined and skipped, -1 = shaken and kept); Q bonds (nqb rows of i, j,
 * cod[ns]); special exclusions (nex rows of i, j, flag[ns]); the Q-Q pairs
 * of the soft-pair list (nsoft rows of iq, jq) for LJ code 2 with qvdw_flag;
 * Q-Q electrostatic scales (nels rows of iq, jq; els_v[nels*ns]).
 * Outputs: qconn[ns][nsol][nq] (int8), per state the nbqq records in the
 * reference's order concatenated (count[s]; iq, j, jq (-1 for a non-Q atom),
 * LJ code, el_scale; capacity cap per state-concatenated arrays), qp_skip[nsol]
 * and the (iq, atom) pairs with qconn(1, atom, iq) == 4 among atoms not
 * skipped, atom-major.  Returns 0, or -1 when cap is too small.
 * ------------------------------------------------------------------------ */
typedef struct {
    int nsol, nq, ns;
    const int *iqatom, *bnd, *qbnd;
    int nb, nqb;
    int8_t *qconn;
} qconn_ctx;

#define QCONN(c, s, i, q) (c)->qconn[((size_t)(s) * (c)->nsol + (i)) * (c)->nq + (q)]

static void find_bonded(qconn_ctx *c, int origin, int current, int level, int state) {
    const int oq = c->iqatom[origin];
    for (int b = 0; b < c->nb; ++b) {
        const int bi = c->bnd[3 * b], bj = c->bnd[3 * b + 1], cod = c->bnd[3 * b + 2];
        if (cod == 0) continue;   /* redefined (but not shaken) */
        int next = -1;
        if (bi == current) next = bj;
        else if (bj == current) next = bi;
        if (next < 0) continue;
        const int nl = level + 1;
        if (QCONN(c, state, next, oq) > nl) {
            QCONN(c, state, next, oq) = (int8_t)nl;
            if (nl < 4) find_bonded(c, origin, next, nl, state);
        }
    }
    const int w = 2 + c->ns;
    for (int b = 0; b < c->nqb; ++b) {
        if (c->qbnd[w * b + 2 + state] <= 0) continue;
        const int bi = c->qbnd[w * b], bj = c->qbnd[w * b + 1];
        int next = -1;
        if (bi == current) next = bj;
        else if (bj == current) next = bi;
        if (next < 0) continue;
        const int nl = level + 1;
        if (QCONN(c, state, next, oq) > nl) {
            QCONN(c, state, next, oq) = (int8_t)nl;
            if (nl < 4) find_bonded(c, origin, next, nl, state);
        }
    }
}

int oracle_qconn(int nsol, int nq, int ns, const int *iqseq, const int *iqatom, const int *iac, const int8_t *ljcod,
                 int natyps, int nb, const int *bnd, int nqb, const int *qbnd, int nex, const int *exspec,
                 int qvdw_flag, int nsoft, const int *soft, int nels, const int *els_ij, const double *els_v,
                 int8_t *qconn, int cap, int *count, int *o_iq, int *o_j, int *o_jq, int *o_lj, double *o_els,
                 uint8_t *qp_skip, int *nqp14, int *qp14) {
    qconn_ctx c = {nsol, nq, ns, iqatom, bnd, qbnd, nb, nqb, qconn};
    memset(qconn, 9, (size_t)ns * nsol * nq);
    for (int iq = 0; iq < nq; ++iq)
        for (int s = 0; s < ns; ++s) QCONN(&c, s, iqseq[iq], iq) = 1;
    for (int iq = 0; iq < nq; ++iq)
        for (int s = 0; s < ns; ++s) find_bonded(&c, iqseq[iq], iqseq[iq], 1, s);
    /* special exclusions: both directions, in the states flagged */
    for (int k = 0; k < nex; ++k) {
        const int *e = exspec + (size_t)k * (2 + ns);
        for (int d = 0; d < 2; ++d) {
            const int a = e[d], other = e[1 - d];
            const int iq = iqatom[a];
            if (iq < 0) continue;
            for (int s = 0; s < ns; ++s)
                if (e[2 + s]) QCONN(&c, s, other, iq) = 0;
        }
    }
    int n = 0;
    for (int s = 0; s < ns; ++s) {
        count[s] = 0;
        /* Q-Q */
        for (int iq = 0; iq < nq - 1; ++iq)
            for (int jq = iq + 1; jq < nq; ++jq) {
                const int j = iqseq[jq];
                const int qc = QCONN(&c, s, j, iq);
                if (qc <= 3) continue;
                if (n >= cap) return -1;
                int lj;
                if (qc == 4) lj = 3;
                else if (!qvdw_flag) lj = ljcod[iac[iqseq[iq]] * natyps + iac[j]];
                else {
                    lj = 1;
                    for (int p = 0; p < nsoft; ++p)
                        if ((iq == soft[2 * p] && jq == soft[2 * p + 1]) || (jq == soft[2 * p] && iq == soft[2 * p + 1])) {
                            lj = 2;
                            break;
                        }
                }
                /* the reference's loop: the first matching entry wins, else 1 */
                double els = 1.0;
                for (int p = 0; p < nels; ++p) {
                    const int k = els_ij[2 * p], l = els_ij[2 * p + 1];
                    if ((iq == k && jq == l) || (iq == l && jq == k)) { els = els_v[(size_t)p * ns + s]; break; }
                }
                o_iq[n] = iq; o_j[n] = j; o_jq[n] = jq; o_lj[n] = lj; o_els[n] = els;
                n++; count[s]++;
            }
        /* Q-non-Q: solute atoms bonded or angled to a Q atom in some state */
        for (int j = 0; j < nsol; ++j) {
            if (iqatom[j] >= 0) continue;
            int near = 0;
            for (int s2 = 0; s2 < ns && !near; ++s2)
                for (int iq = 0; iq < nq; ++iq)
                    if (QCONN(&c, s2, j, iq) <= 3) { near = 1; break; }
            if (!near) continue;
            for (int iq = 0; iq < nq; ++iq) {
                const int qc = QCONN(&c, s, j, iq);
                if (qc < 4) continue;
                if (n >= cap) return -1;
                o_iq[n] = iq; o_j[n] = j; o_jq[n] = -1;
                o_lj[n] = qc == 4 ? 3 : (qvdw_flag ? 1 : ljcod[iac[iqseq[iq]] * natyps + iac[j]]);
                o_els[n] = 1.0;
                n++; count[s]++;
            }
        }
    }
    /* nbqplist's skips (:10288) and 1-4 codes from state 1 (:10306) */
    int np = 0;
    for (int j = 0; j < nsol; ++j) {
        int skip = 0;
        for (int s = 0; s < ns && !skip; ++s)
            for (int iq = 0; iq < nq; ++iq)
                if (QCONN(&c, s, j, iq) <= 3) { skip = 1; break; }
        qp_skip[j] = (uint8_t)skip;
        if (skip) continue;
        for (int iq = 0; iq < nq; ++iq)
            if (QCONN(&c, 0, j, iq) == 4) {
                if (np >= cap) return -1;
                qp14[2 * np] = iq; qp14[2 * np + 1] = j;
                np++;
            }
    }
    *nqp14 = np;
    return 0;
}
