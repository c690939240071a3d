/*
 * qgpu.h -- C-ABI of the GB300 engine for the hot path of Q's qdyn.
 *
 * The reference (qusers/qsource, Q 5.06) is Fortran 90.  Its hot path lives in
 * src/md.f90 as zero-argument module subroutines that read and write module
 * globals.  This header replaces those call points with plain C entry points:
 * every array is a plain pointer plus a size, no torch or CUDA types appear,
 * and every call returns an int status (0 = ok, see QGPU_E_*).  The text of the
 * last error is returned by qgpu_last_error().
 *
 * Conventions
 *   - Atom, group, Q-atom and type indices are 0-based (the Fortran host
 *     subtracts 1 once when it fills the descriptor).
 *   - Coordinates, velocities and forces are interleaved xyz FP64 arrays of
 *     length 3*natom, the layout of md.f90's x(:), v(:), d(:) (src/md.f90:309-313).
 *   - Charges are already multiplied by sqrt(coulomb_constant), as prep_sim does
 *     (src/md.f90:16805-16811), so q_i*q_j/r is in kcal/mol.
 *   - dt and tau_T are in Q's internal time unit (0.020462 * fs,
 *     src/md.f90:4623,4637).
 *
 * A handle holds a batch of ntraj independent trajectories (lambda windows or
 * replicas).  ntraj == 1 is the drop-in mode that sits behind one qdyn
 * process; ntraj > 1 is the batched mode that runs many windows in one
 * launch sequence.
 */
#ifndef QGPU_H
#define QGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QGPU_MAX_STATES 10   /* max_states, src/qatom.f90:37 */

/* status codes */
#define QGPU_OK               0
#define QGPU_E_INVALID        1   /* bad descriptor / argument */
#define QGPU_E_CUDA           2   /* CUDA runtime error */
#define QGPU_E_LIST_OVERFLOW  3   /* a neighbour list ran out of capacity */
#define QGPU_E_SHAKE          4   /* SHAKE did not converge in SHAKE_MAX_ITER */
#define QGPU_E_NAN            5   /* non-finite temperature (md.f90:6654-6656) */
#define QGPU_E_UNSUPPORTED    6   /* input uses a feature this engine does not run */
#define QGPU_E_FIXED_RANGE    7   /* a fixed-point accumulator left its range */

/* ------------------------------------------------------------------------ */
/* System descriptor: the qdyn module state after topology/prep_coord/get_fep/ */
/* prep_sim/init_shake/make_nbqqlist/shrink_topology (src/qdyn.f90:110-124).  */
/* ------------------------------------------------------------------------ */
typedef struct qgpu_system_desc {
    /* sizes */
    int32_t natom;          /* nat_pro                                         */
    int32_t nat_solute;     /* solute atoms come first, waters after           */
    int32_t solv_atom;      /* atoms per solvent molecule; must be 3           */
    int32_t nwat;           /* (natom - nat_solute) / solv_atom               */
    int32_t natyps;         /* atom types                                      */
    int32_t ncgp;           /* charge groups (solute groups first)             */
    int32_t ncgp_solute;
    int32_t nqat;           /* Q atoms                                         */
    int32_t nstates;        /* FEP/EVB states (<= QGPU_MAX_STATES)             */

    /* coordinates */
    const double *x;        /* 3*natom starting coordinates                    */
    const double *v;        /* 3*natom starting velocities (may be NULL)       */
    const double *xtop;     /* 3*natom topology coordinates (restraint origin) */

    /* per atom */
    const double  *crg;     /* natom, scaled charges                           */
    const int32_t *iac;     /* natom, atom type                                */
    const uint8_t *excl;    /* natom, atom outside the sphere (excluded)       */
    const uint8_t *shell;   /* natom, atom in the restrained shell             */
    const int32_t *iqatom;  /* natom, Q-atom index or -1                       */

    /* atom-type library (iaclib) and LJ code matrix (ljcod) */
    const double *mass;     /* natyps                                          */
    const double *avdw;     /* natyps*3, [type*3 + (ljcode-1)]                 */
    const double *bvdw;     /* natyps*3                                        */
    const int8_t *ljcod;    /* natyps*natyps, values 1 or 2                    */
    double el14_scale;
    int32_t ivdw_rule;      /* 1 geometric, 2 arithmetic (nonbon2_*)           */
    int32_t ff_type;        /* 1 GROMOS, 2 AMBER, 3 CHARMM (improper form)     */

    /* SPC-type solvent tables (prep_sim, src/md.f90:16702-16717) */
    double chg_solv[3];     /* scaled charges of the 3 solvent atoms           */
    double aLJ_solv[6];     /* [atom*2 + (ljcode-1)]                           */
    double bLJ_solv[6];

    /* charge groups */
    const int32_t *cgp_first;   /* ncgp, index into cgpatom                    */
    const int32_t *cgp_last;    /* ncgp, inclusive                             */
    const int32_t *cgp_switch;  /* ncgp, switch atom                           */
    const int32_t *cgpatom;     /* natom                                       */

    /* solute neighbour exclusions and 1-4 pairs (listex/listexlong and
       list14/list14long merged), each pair stored once with i < j */
    int32_t nexcl;  const int32_t *excl_pairs;   /* 2*nexcl */
    int32_t n14;    const int32_t *pairs14;      /* 2*n14   */

    /* Q atoms (src/qatom.f90, get_fep src/md.f90:2884-3074) */
    const int32_t *iqseq;       /* nqat, atom of each Q atom                   */
    const double  *qcrg;        /* nqat*nstates [iq*nstates+s], scaled         */
    int32_t qvdw_flag;          /* Q atoms have their own LJ types per state   */
    const int32_t *qiac;        /* nqat*nstates, Q-type per state              */
    int32_t nqlib;              /* Q atom types                                */
    const double  *qavdw;       /* nqlib*3                                     */
    const double  *qbvdw;       /* nqlib*3                                     */
    const double  *sc_lookup;   /* nqat*(natyps+nqat)*nstates, softcore shifts  */
                                /* [(iq*(natyps+nqat) + col)*nstates + s]      */
    double lambda[QGPU_MAX_STATES];

    /* Q-atom / solute list inputs that make_qconn derives at start-up       */
    const uint8_t *qp_skip;     /* natom: any(qconn(:,i,:) <= 3)  (md.f90:10288) */
    int32_t nqp14;  const int32_t *qp14_pairs; /* 2*n: (iq, atom) with qconn(1,atom,iq)==4 */

    /* nbqqlist (src/md.f90:9691-9804), per state, concatenated               */
    int32_t nbqq_count[QGPU_MAX_STATES];
    const int32_t *nbqq_iq;     /* sum(nbqq_count) entries                     */
    const int32_t *nbqq_j;      /* atom                                        */
    const int32_t *nbqq_jq;     /* Q atom of j or -1                           */
    const int8_t  *nbqq_ljcod;
    const double  *nbqq_elscale;

    /* Q bonded terms (per-state codes, 0 = absent in that state) */
    int32_t nqbond;  const int32_t *qbnd;      /* nqbond*(2+nstates): i, j, cod[s] (1-based codes) */
    int32_t nqbcod;  const double  *qbondlib;  /* nqbcod*4: Dmz, amz, r0, fk                      */
    int32_t nqangle; const int32_t *qang;      /* nqangle*(3+nstates)                              */
    int32_t nqacod;  const double  *qanglib;   /* nqacod*4: fk, ang0 (rad), ureyfk, ureyr0         */
    int32_t nqtor;   const int32_t *qtor;      /* nqtor*(4+nstates)                                */
    int32_t nqtcod;  const double  *qtorlib;   /* nqtcod*3: fk, rmult, deltor (rad)                */
    int32_t nqimp;   const int32_t *qimp;      /* nqimp*(4+nstates)                                */
    int32_t nqicod;  const double  *qimplib;   /* nqicod*2: fk, imp0 (rad)                         */

    /* classical bonded terms after shrink_topology (codes 1-based) */
    int32_t nbonds, nbonds_solute;  const int32_t *bnd;   /* nbonds*3: i, j, cod   */
    int32_t nbndcod;  const double *bondlib;               /* nbndcod*2: fk, b0     */
    int32_t nangles, nangles_solute; const int32_t *ang;   /* nangles*4             */
    int32_t nangcod;  const double *anglib;                /* nangcod*4: fk, ang0 (rad), ureyfk, ureyr0 */
    int32_t ntors, ntors_solute;    const int32_t *tor;    /* ntors*5               */
    int32_t ntorcod;  const float  *torlib;                /* ntorcod*4: fk, rmult, deltor (rad), 1/paths (single, as topo.f90) */
    int32_t nimps, nimps_solute;    const int32_t *imp;    /* nimps*5               */
    int32_t nimpcod;  const float  *implib;                /* nimpcod*2: fk, imp0 (rad) */

    /* SHAKE (init_shake, src/md.f90:4242-4426), molecules in CSR form */
    int32_t shake_molecules;
    const int32_t *shake_first; /* shake_molecules+1                           */
    const int32_t *shake_i;     /* constraint atoms                            */
    const int32_t *shake_j;
    const double  *shake_dist2; /* squared target distance                     */

    /* off-diagonal EVB couplings: Hij = A*exp(-mu*r_kl) (src/md.f90:15444) */
    int32_t noffd;
    const int32_t *offd_ij;     /* noffd*2 states                              */
    const int32_t *offd_kl;     /* noffd*2 Q atoms                             */
    const double  *offd_Amu;    /* noffd*2: A, mu                              */

    /* simulation sphere (topology + [sphere]/[solvent] sections) */
    double xpcent[3];           /* solute centre                               */
    double xwcent[3];           /* solvent centre                              */
    double rexcl_o;             /* exclusion radius                            */
    double rwat;                /* water sphere radius                         */
    double fk_wsphere, Dwmz, awmz;   /* radial solvent restraint               */
    double fk_pshell, fk_fix;   /* shell / excluded atom restraints            */
    int32_t wpol_restr;         /* water polarisation restraint requested       */

    /* cut-offs ([cut-offs]) */
    double Rcpp, Rcww, Rcpw, Rcq, RcLRF;
    int32_t use_LRF;

    /* MD parameters ([MD]) */
    double dt;                  /* internal units                              */
    double Temp0, tau_T;        /* tau_T in internal units                     */
    int32_t separate_scaling;
    int32_t NBcycle;
    int32_t Ndegf, Ndegfree, Ndegf_solvent, Ndegfree_solvent;
    int32_t Ndegf_solute, Ndegfree_solute, detail_temps;

    /* list variant: 0 = switch-atom cut-off (topology flag iuse_switch_atom = 1,
       nbpplist_lrf/nbpwlist_lrf/nbqplist); 1 = any-atom cut-off for solute
       groups (iuse_switch_atom = 0, nbpplis2_lrf src/md.f90:7441,
       nbpwlis2_lrf :8902, nbqplis2 :9946) */
    int32_t any_atom_lists;

    /* sequence restraints ([sequence_restraints], p_restrain src/md.f90:15484-15576) */
    int32_t nrstr_seq;
    const int32_t *rstseq_ij;     /* 2*n: first, last atom (inclusive)                */
    const double  *rstseq_fk;     /* n: force constant                                */
    const int32_t *rstseq_flags;  /* 2*n: ih (1 = hydrogens too), to_centre (0 each   */
                                  /*      atom, 1 geometric centre, 2 mass centre)    */
    const uint8_t *heavy;         /* natom: mass >= 4 (topo.f90:871-880)              */
    int32_t excluded_freeze;      /* [sphere] excluded_freeze                         */

    /* water polarisation restraint (watpol src/md.f90:18372-18541; the shells of
       wat_shells :18185-18368, used when wpol_restr != 0) */
    double fkwpol;
    int32_t nwpolr_shell;
    const double *wshell_rout;    /* nwpolr_shell: outer radius                       */
    const double *wshell_dr;      /* nwpolr_shell: width                              */
    const double *wshell_cstb;    /* nwpolr_shell: Born term                          */
    const double *wshell_theta_corr; /* nwpolr_shell: starting theta_corr (restart) */
    int32_t itdis_update;         /* theta_corr update interval (100)                 */

    /* thermostat and integrator ([MD], md_run src/md.f90:6440-6460, 6577-6606) */
    int32_t thermostat;           /* 0 Berendsen, 1 Langevin, 2 Nose-Hoover           */
    int32_t integrator;           /* 0 leap-frog, 1 velocity-verlet                   */
    double friction;              /* Langevin friction (internal time units^-1)       */
    int32_t langevin_gauss;       /* Langevin random forces: 0 uniform, 1 Gaussian    */
    int32_t rand_state;           /* randm state (iseed) when the run starts           */
    int32_t nhchains;             /* Nose-Hoover chain length                         */
    double nhq;                   /* Nose-Hoover mass                                 */

    /* periodic box: topology boundary record "PBC" (topo_read src/topo.f90:
       1022-1031), [PBC] of the input (initialize src/md.f90:4514-4590) and of
       the FEP file (switching_atom, src/qatom.f90:672-687).  use_pbc = 0 is the
       simulation sphere and the fields below are ignored.  With use_pbc = 1
       the lists and pair loops take minimum images (make_pair_lists box branch
       src/md.f90:6003-6029, pot_energy_nonbonds :16266-16300); the sphere
       restraints (fix_shell, restrain_solvent, watpol) are off (:16114-16124). */
    int32_t use_pbc;
    double boxlength[3];
    double boxcentre[3];
    int32_t qswitch;              /* Q-atom switching atom, 0-based (PBC with Q atoms) */
    int32_t put_solute_back;      /* put_back_in_box of solute molecules              */
    int32_t put_solvent_back;     /* put_back_in_box of solvent molecules             */
    int32_t rigid_box_centre;     /* 0: box centre follows the solute (put_back_in_box)*/
    int32_t nmol;                 /* molecules                                        */
    const int32_t *istart_mol;    /* nmol: first atom of each molecule, 0-based       */
    int32_t nsolute_mol;          /* the first nsolute_mol molecules are solute       */

    /* the other restraints of p_restrain (src/md.f90:15580-15800; input
       initialize :5234-5358).  state: 0 = every state (energy into each
       state's restraint term), s >= 1 = that state only, its force weighted by
       lambda_s.  Wall restraints (sphere only) act on the atoms first..last
       that are heavy or, with the H flag, any atom. */
    int32_t nrstr_pos;  const int32_t *rstpos_i;  /* 2n: atom, state                  */
    const double *rstpos_x;                         /* 6n: x0[3], fk[3]                 */
    int32_t nrstr_dist; const int32_t *rstdis_i;  /* 3n: atom i, atom j, state        */
    const double *rstdis_p;                         /* 3n: d1, d2, fk                   */
    int32_t nrstr_angl; const int32_t *rstang_i;  /* 4n: atoms i, j, k, state         */
    const double *rstang_p;                         /* 2n: angle (degrees), fk          */
    int32_t nrstr_wall; const int32_t *rstwal_i;  /* 3n: first, last atom, H flag     */
    const double *rstwal_p;                         /* 4n: d, fk, aMorse, dMorse        */
} qgpu_system_desc;

/* Energies, the ENERGIES record of src/nrgy.f90:48-54 (sphere subset). */
typedef struct qgpu_energies {
    double potential, kinetic, lrf;
    double p_bond, p_angle, p_torsion, p_improper;
    double w_bond, w_angle, w_torsion, w_improper;
    double q_bond, q_angle, q_torsion, q_improper;
    double pp_el, pp_vdw, pw_el, pw_vdw, ww_el, ww_vdw, qx_el, qx_vdw;
    double rst_total, rst_fix, rst_shell, rst_protein, rst_solvent_radial, rst_water_pol;
} qgpu_energies;

/* Per-state Q energies, the Q_ENERGIES record of src/nrgy.f90:56-63 with
   one group-contribution array (arrays = 1). */
typedef struct qgpu_qenergy {
    double lambda;
    double q_bond, q_angle, q_torsion, q_improper;
    double qq_el, qq_vdw, qp_el, qp_vdw, qw_el, qw_vdw, qx_el, qx_vdw;
    double restraint, total;
} qgpu_qenergy;

/* Which terms qgpu_forces evaluates.  The drop-in split keeps restraints and
   classical bonded terms on the host (pot_energy, src/md.f90:16100-16150);
   the persistent run mode needs all of them on the device. */
#define QGPU_TERMS_NONBOND   0x1   /* pot_energy_nonbonds: pp pw qp ww qw + LRF */
#define QGPU_TERMS_QQ        0x2   /* nonbond_qq                                 */
#define QGPU_TERMS_QBONDED   0x4   /* qbond/qangle/qtorsion/qimproper            */
#define QGPU_TERMS_BONDED    0x8   /* pot_energy_bonds                           */
#define QGPU_TERMS_RESTRAINT 0x10  /* fix_shell + restrain_solvent               */
#define QGPU_TERMS_ALL       0x1f
/* Flag for qgpu_forces: evaluate with the precision of an MD step whose
   energies are not recorded (FP32 throughout, energies from FP32 sums)
   instead of the FP64 energies of the drop-in call. */
#define QGPU_TERMS_STEP_PRECISION 0x100

typedef struct qgpu_handle qgpu_handle;

/* Energy sink for qgpu_run_block: called on the host after the block with
   one row per (trajectory, recorded step). */
typedef void (*qgpu_ene_sink)(void *user, int32_t traj, int32_t step,
                              const qgpu_qenergy *eq, int32_t nstates,
                              const qgpu_energies *e);

/* ---- lifetime ----------------------------------------------------------- */
/* Copies the descriptors to the device.  Replaces the data set-up that the
   qdyn master performs before md_run (src/qdyn.f90:110-137).  descs[t]
   describes trajectory t; the host keeps ownership of its arrays. */
int qgpu_create(const qgpu_system_desc *descs, int32_t ntraj, qgpu_handle **out);
int qgpu_destroy(qgpu_handle *h);
int qgpu_last_error(char *buf, int32_t len);
int qgpu_ntraj(const qgpu_handle *h);

/* ---- state transfer ----------------------------------------------------- */
int qgpu_set_coords(qgpu_handle *h, int32_t traj, const double *x, const double *v);
int qgpu_get_coords(qgpu_handle *h, int32_t traj, double *x, double *v);
/* The same for every trajectory of the batch at once: x and v hold the
   trajectories' 3*natom arrays back to back in trajectory order (one copy
   each way instead of one per trajectory). */
int qgpu_set_coords_all(qgpu_handle *h, const double *x, const double *v);
int qgpu_get_coords_all(qgpu_handle *h, double *x, double *v);

/* ---- drop-in call points ------------------------------------------------ */
/* make_pair_lists (src/md.f90:5985-6071): group centres, pp/pw/ww lists with
   LRF multipoles for pairs beyond the cut-offs, and (first call only, as the
   reference with Rcq > rexcl_o) the qp and qw lists.  All trajectories. */
int qgpu_build_lists(qgpu_handle *h);

/* pot_energy (src/md.f90:16015-16221) restricted to `terms`: forces d (3N,
   may be NULL), energies E and per-state EQ[nstates] (may be NULL) of
   trajectory traj.  Evaluates every trajectory; copies back one. */
int qgpu_forces(qgpu_handle *h, int32_t traj, int32_t terms,
                double *d, qgpu_energies *E, qgpu_qenergy *EQ);

/* shake (src/md.f90:17581-17679) on trajectory traj: xx = coordinates before
   the update, x = after; x is corrected in place.  niter = average
   iterations per molecule, as the reference returns. */
int qgpu_shake(qgpu_handle *h, int32_t traj, const double *xx, double *x, int32_t *niter);

/* ---- persistent mode ---------------------------------------------------- */
/* Runs nsteps MD steps of every trajectory on the device (Berendsen leap-frog,
   SHAKE, lists every NBcycle), each NBcycle-step block replayed from a CUDA
   graph.  Energies of every `ene_every`-th step are collected on the device
   and handed to `sink` after the block (sink may be NULL). */
int qgpu_run(qgpu_handle *h, int32_t nsteps, int32_t ene_every,
             qgpu_ene_sink sink, void *user);
/* qgpu_run with the energy records written to host arrays instead of a
   callback (a Fortran host's put_ene loop reads them in bulk): row r is
   E_rows[r], EQ_rows[r*QGPU_MAX_STATES ...], step_rows[r], traj_rows[r], in
   the order qgpu_run's sink would see them; at most cap rows, *nrows gets the
   count written (rows beyond cap are dropped, *nrows says how many came). */
int qgpu_run_rows(qgpu_handle *h, int32_t nsteps, int32_t ene_every, qgpu_energies *E_rows,
                  qgpu_qenergy *EQ_rows, int32_t *traj_rows, int32_t *step_rows, int32_t cap, int32_t *nrows);

/* Autotuner.  Times every launch shape of the pair kernels on this handle's
   own lists -- lanes per target water (4/8/16), the water kernel's register
   bound (1 or 6 resident blocks) and neighbours per loop iteration (1/2/4; 3: a software
   pipeline, one neighbour per iteration with the next one's loads in flight),
   lanes per Q-water item (1/2/4), lanes per solute atom (4/8/16) -- keeps the
   fastest, and caches the choice per device and system size for later
   handles of the process.  tuning[5] (may be NULL) receives {lanes_water,
   min_blocks_water, lanes_solute, lanes_qw, unroll_water}.  Results are deterministic for a given choice;
   different choices sum the float pair terms in a different order. */
int qgpu_autotune(qgpu_handle *h, int32_t *tuning);
/* Pins a choice (the values qgpu_autotune reports; lanes_qw 0 = by Q count). */
int qgpu_set_tuning(qgpu_handle *h, const int32_t *tuning);

/* Sets the step counter istep (md_run's loop index).  The water polarisation
   restraint updates its theta_corr when istep is a nonzero multiple of
   itdis_update (src/md.f90:18451); qgpu_run advances the counter itself, a
   drop-in host that calls qgpu_forces once per step sets it before each call. */
int qgpu_set_step(qgpu_handle *h, int64_t istep);

/* Precision of the persistent MD step (qgpu_run / qgpu_enqueue).
   QGPU_PRECISION_FP64 (the default): FP64 master x and v with the
     reference's FP64 leap-frog / velocity-Verlet and thermostat updates
     (newvel_ber, src/md.f90:6194-6223; newvel_lan, newvel_nos), FP64 SHAKE
     (src/md.f90:17581-17679) and FP64 temperatures and Berendsen scales
     (temperature, src/md.f90:6098-6190, from exact integer sums of the
     per-atom kinetic energies) every step.  When every trajectory's
     constraints are 3-site waters (O-H, O-H, H-H) the update, SHAKE and the
     step's end run as one fused kernel; otherwise as separate kernels.
   QGPU_PRECISION_FP64_UNFUSED: the same FP64 arithmetic in the separate
     update, SHAKE and step-end kernels whatever the constraints.
   QGPU_PRECISION_MIXED: master positions as a double-float (about 48
     significant bits), FP32 velocities, SHAKE of 3-site waters in FP32 on
     relative vectors, FP32 temperature, FP32 bonded/restraint terms on
     unrecorded steps; FP64 energies on recorded steps.  Used when every
     trajectory's constraints are 3-site waters, else the FP64 form runs.
   Pair terms are FP32 with int64 fixed-point sums in every mode.  Switching
   keeps the current coordinates and velocities. */
/* Concurrency of a batch's replayed 10-step blocks (qgpu_run /
   qgpu_enqueue with the fused step forms): the trajectories are split into
   at most n groups of consecutive trajectories with about equal atom counts
   (1 <= n <= 8; default 4), and each group's list build
   and steps form an independent branch of the block's CUDA graph, so that one
   group's FP64 update (FP64-unit bound) runs beside another group's force
   kernels (FP32 and memory bound).  Results do not depend on n: every
   trajectory's arithmetic is the same.  qgpu_get_branches returns the number
   of groups in use. */
int qgpu_set_branches(qgpu_handle *h, int32_t n);
int qgpu_get_branches(const qgpu_handle *h);

#define QGPU_PRECISION_MIXED 0
#define QGPU_PRECISION_FP64  1
#define QGPU_PRECISION_FP64_UNFUSED 2
int qgpu_set_precision(qgpu_handle *h, int32_t mode);

/* Queues nsteps of the same device work as qgpu_run without waiting for it
   (no energy sink); a failure surfaces at the next qgpu_sync or qgpu_run. */
int qgpu_enqueue(qgpu_handle *h, int32_t nsteps, int32_t ene_every);
/* Waits for all queued work of the handle and returns its status. */
int qgpu_sync(qgpu_handle *h);

/* ---- energy files and free energies ------------------------------------- */
/* Attaches a Q energy file (.en, the layout of put_ene, src/nrgy.f90:94-123,
   with the header of src/md.f90:17011-17015; arrays = 1) to trajectory traj:
   writes the header now and, during qgpu_run, one frame for every recorded
   step > 0, as qdyn does every iene_cycle steps (md_run :6630-6633).  qfep
   reads these files unchanged. */
int qgpu_ene_open(qgpu_handle *h, int32_t traj, const char *path);
int qgpu_ene_close(qgpu_handle *h, int32_t traj);
/* Writes a whole energy file from host rows: nframes frames of nstates
   qgpu_qenergy each, with noffd couplings per frame (offd_ij: 1-based state
   pairs, offd_Hr: nframes*noffd (Hij, rkl)).  No device involved. */
int qgpu_enefile_write(const char *path, int32_t nframes, int32_t nstates, const qgpu_qenergy *frames,
                       int32_t noffd, const int32_t *offd_ij, const double *offd_Hr);

/* qfep's input (src/qfep.f90:110-230), in the order it reads it. */
#define QGPU_QFEP_MAXCOUP 45                       /* state pairs of QGPU_MAX_STATES states */
#define QGPU_QFEP_P2 (5 + QGPU_MAX_STATES)          /* doubles per Part 2 row */
#define QGPU_QFEP_P3 7                              /* doubles per Part 3 row */
typedef struct {
    int32_t nstates;      /* states per frame */
    int32_t noffd;        /* off-diagonal elements stored in the files ("predefined") */
    double kT;
    int32_t nskip;        /* frames skipped at the start of every file */
    int32_t gas;          /* 1: V_s = Q bonded + qq (el + vdW) + restraint ("calculation mode") */
    int32_t nbins;        /* energy-gap bins */
    int32_t nmin;         /* minimum points per bin (>= 1) */
    double alpha[QGPU_MAX_STATES];  /* shift of each state's energy; alpha[0] is taken as 0 */
    double scale_hij;     /* noffd > 0: Hij(1,2) = scale_hij * the file's Hij when > 0 (two states) */
    int32_t ncoup;        /* noffd == 0: couplings Hij = A exp(-mu (r - r0)) exp(-eta (r - r0)^2),
                             r = the first file coupling's distance; the files then hold ncoup
                             off-diagonal entries per frame */
    int32_t coup_ij[2 * QGPU_QFEP_MAXCOUP];       /* 1-based state pairs */
    double coup_A[QGPU_QFEP_MAXCOUP], coup_mu[QGPU_QFEP_MAXCOUP], coup_eta[QGPU_QFEP_MAXCOUP],
        coup_rxy0[QGPU_QFEP_MAXCOUP];
    double coeff[QGPU_MAX_STATES];  /* reaction coordinate: gap = sum_s coeff[s] (V_s + alpha[s]) */
} qgpu_qfep_params;
/* qfep Parts 1-3 (src/qfep.f90:416-835) on nfiles energy files in lambda
   order, host code.  Per frame the state energies are shifted by alpha, the
   EVB ground state Eg is the lowest eigenvalue of H (H_ii = V_i, H_ij the
   coupling; two states: the closed form of qfep with the mixing c1 = 1/(1 +
   ((Eg - V_1)/H_12)^2), c2 = 1 - c1), the gap is sum_s coeff_s V_s.
     part1[3 w + 0..2]: dGf(w) (0 for the last window), dGr(w) (0 for the
       first), dG(w) (Part 1);
     gaprange[2]: smallest and largest gap over the frames after nskip;
     part2[(w nbins + b) QGPU_QFEP_P2]: window w, bin b: points, gap at the
       bin centre, dGg (ground state), <c1>, <c2>, dGv_1 .. dGv_nstates
       (diabatic curves); values are written where points >= nmin, else 0;
     part3[b QGPU_QFEP_P3]: points over all windows, gap, <dGg>, <dGg> - min,
       <c1>, <c2>, <r_xy> of the bin (values where points >= nmin);
       min is qfep's: over every bin's sum including empty ones (0);
     npts[w]: frames read from file w.
   Returns QGPU_E_INVALID for unreadable files, bad parameters or a zero gap
   range. */
int qgpu_qfep_evb(int32_t nfiles, const char *const *paths, const qgpu_qfep_params *p, double *part1,
                  double *gaprange, double *part2, double *part3, int32_t *npts);
/* Free-energy perturbation over a chain of lambda windows, accumulated on
   the device from every recorded frame with a nonzero step (qfep Part 1,
   src/qfep.f90:609-661): window w = trajectory chain[w]; per frame
   dv = sum_s lambda_{w+-1,s} V_s - sum_s lambda_{w,s} V_s with V_s the state
   total, and the sums of exp(-dv/kT) (FP64, in frame order) and of dv, dv^2,
   dv^3 per direction; the first nskip frames of each window are skipped.
   Starting clears the sums. */
int qgpu_fep_start(qgpu_handle *h, int32_t nwin, const int32_t *chain, double kT, int32_t nskip);
/* qfep's dgf(w) = -kT ln<exp(-dv_f/kT)> (w < nwin-1), dgr(w) (w > 0) and
   dG(w) = dG(w-1) + (dgf(w-1) - dgr(w))/2, dG(0) = 0, each nwin long; stats
   (may be NULL) gets 7 values per window: frames, mean / variance / skew of
   dv forward, and of dv backward. */
int qgpu_fep_result(qgpu_handle *h, double *dgf, double *dgr, double *dg, double *stats);

/* ---- learned lambda schedule: the MLP ----------------------------------- */
/* Has no counterpart in the reference (qdyn runs lambda windows one after
   another on a fixed schedule).  A 3-layer MLP, 16 inputs (zero-padded) ->
   tanh 128 -> tanh 128 -> 1, run by hand-written one-block kernels whose
   layer products use BF16 tensor-core mma with FP32 accumulation; FP32 master
   parameters, Adam moments.  Parameter layout (floats): W1[128][16], b1[128],
   W2[128][128], b2[128], W3[16][128] (row 0 used), b3[16] (entry 0 used);
   qgpu_mlp_nparams() floats in all.  Batches hold 1..64 rows of 16 features. */
int qgpu_mlp_nparams(void);
/* out[n] = network(X[n][16]) */
int qgpu_mlp_predict(const float *params, const float *X, int32_t n, float *out);
/* iters full-batch Adam steps (lr; beta 0.9/0.999) on the mean squared error
   to Y[n], deterministic; params, adam_m, adam_v updated in place; step0 =
   Adam steps already taken; loss_out[iters] (may be NULL) the loss before each
   step; grad_out[nparams] (may be NULL) the gradient of the last step. */
int qgpu_mlp_train(float *params, float *adam_m, float *adam_v, const float *X, const float *Y, int32_t n,
                   int32_t iters, float lr, int32_t step0, float *loss_out, float *grad_out);

/* ---- inspection (tests and tools) --------------------------------------- */
/* Near charge-group pairs of the last list build, one row per unordered pair
   (g1 < g2), with g1,g2 0-based group indices.  Returns the count in *npairs;
   rows are written only if cap >= count. */
int qgpu_get_group_pairs(qgpu_handle *h, int32_t traj, int32_t *pairs, int64_t cap, int64_t *npairs);
/* Q-atom lists of the last list build (nbqplist / nbqplis2 / nbqplist_box,
   src/md.f90:10215, :9946, :10327; nbqwlist / nbqwlist_box, :10464, :10554):
   the solute atoms paired with every Q atom (0-based atom indices, ascending;
   atoms that nbqplist skips, :10288, are absent) and the waters paired with
   every Q atom (their O atoms, ascending).  Counts in *nqp / *nqw; rows are
   written up to cap_qp / cap_qw. */
int qgpu_get_q_lists(qgpu_handle *h, int32_t traj, int32_t *qp_atoms, int64_t cap_qp, int64_t *nqp,
                     int32_t *qw_waters, int64_t cap_qw, int64_t *nqw);
/* LRF records of the last list build: ncgp rows of 3 centre + 1 + 3 + 9 + 27
   doubles (cgp_cent, phi0, phi1, phi2, phi3), the LRF_TYPE of md.f90:444-450. */
int qgpu_get_lrf(qgpu_handle *h, int32_t traj, double *lrf43);
/* Last temperature record: Temp, Tfree, Tscale_solute, Tscale_solvent. */
int qgpu_get_temperature(qgpu_handle *h, int32_t traj, double *out4);
/* Kernel launches issued by the library since creation. */
int64_t qgpu_kernel_launches(const qgpu_handle *h);
/* The CUDA stream (cudaStream_t) all of this handle's work runs on, so a
   caller can order its own work or record timing events against it. */
void *qgpu_stream(qgpu_handle *h);
/* Runs nsteps MD steps kernel by kernel with CUDA events around each launch;
   per distinct kernel: name (64-char slots in names), total ms, launches. */
int qgpu_profile(qgpu_handle *h, int32_t nsteps, char *names, double *ms, int64_t *counts, int32_t cap,
                 int32_t *nkernels);
/* Measured FP32 FMA throughput of the device in TFLOP/s (an FMA-chain kernel
   over all SMs, timed with CUDA events); the roofline denominator of the
   FP32-bound pair and LRF kernels. */
int qgpu_fp32_peak(double *tflops);
/* FP64 FMA throughput of the current device in TFLOP/s (independent DFMA
   chains on every SM), the denominator of the FP64 update's roofline. */
int qgpu_fp64_peak(double *tflops);
/* SHAKE work since the last call, over all trajectories: molecule sweeps
   (every step form) and constraint visits (the FP64 fused step); the
   counters are reset. */
int qgpu_shake_counts(qgpu_handle *h, int64_t *sweeps, int64_t *visits);

/* ---- allocation-free scan ----------------------------------------------- */
/* Has no counterpart in the reference.  For callers that may not allocate
   device memory -- a host program whose device memory belongs to its own
   allocator or to a pool reserved once at start-up, or a time-step loop in
   which a cudaMalloc (which can synchronise the device) is not allowed: the
   charge-group scan of qgpu_build_lists (switch-atom cut-off, topology flag
   iuse_switch_atom = 1) for ONE system, on arrays the caller
   already holds on the device, with no engine handle.  It allocates nothing:
   its chunk partials live in a fixed 8 MiB device array of the library, held
   by every device that loads it until the process exits.
     inputs (device): x[3*natom] coordinates; crg[natom] scaled charges, 0 for
       atoms that must not feed the multipoles (Q atoms); g_start[ngroup+1] and
       g_atoms[] the members of each charge group (0-based atoms); g_switch
       [ngroup] the switch atom; g_flags[ngroup] bit 0 = solvent group, bit 1 =
       excluded group.  origin (host, 3 doubles): the point the float
       coordinates are taken relative to (the solvent sphere centre).
     cut-offs: rc_pp, rc_pw, rc_ww (near groups), rc_lrf (multipole range).
     outputs (device): lrf43[ngroup*43] in the layout of qgpu_get_lrf;
       near_count[ngroup] the number of groups inside the cut-off.
   Limit: ngroup <= 65536; larger systems are refused with QGPU_E_INVALID.
   The first call on each device resolves the array's device address (with
   that device current); make it before any stream capture.  Work is queued on
   `stream` (a cudaStream_t, NULL = legacy default stream) and the call returns
   without waiting.  All calls share the one array: two calls whose work
   overlaps on the GPU (other streams, other host threads) race on it. */
int qgpu_lrf_scan_static(int32_t ngroup, const double *x, const double *crg, const int32_t *g_start,
                         const int32_t *g_atoms, const int32_t *g_switch, const int32_t *g_flags,
                         const double *origin, double rc_pp, double rc_pw, double rc_ww, double rc_lrf,
                         double *lrf43, int32_t *near_count, void *stream);

/* ------------------------------------------------------------------------ */
/* qcalc-style trajectory analysis (src/qcalc.f90 and its calc_* modules) on  */
/* the device.  frames: nframes x 3*natom FP64 coordinates in host memory     */
/* (e.g. the frames of a DCD trajectory, src/trj.f90), uploaded once per call;*/
/* every calculation runs over all frames in one launch.  Atom indices are    */
/* 0-based; masks are atom lists in topology order.                           */
/* ------------------------------------------------------------------------ */
/* RMS deviation of the masked atoms from xref (3*natom, the topology
   coordinates in qcalc), no fitting: sqrt(sum |x - x0|^2 / nmask)
   (calc_rms.f90 rms_calc).  out[nframes], A. */
int qgpu_calc_rms(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                  const double *xref, double *out);
/* RMS fluctuation of the masked atoms (calc_rmsf.f90 RMSF_calc): after each
   frame, per atom sqrt(mean of |x|^2 - |running mean of x|^2) over the frames
   so far (the reference's running-mean update), averaged over the mask.
   out[nframes], A: the value qcalc prints at each frame. */
int qgpu_calc_rmsf(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                   double *out);
/* Least-squares fit (calc_fit.f90 fit_calc, LSQSTR): every frame's solute
   atoms (the first nsol) superposed on the topology coordinates xref by the
   mass-weighted fit of the masked atoms (mask: solute atom indices), the
   rotation from the eigenvectors of [[0, U], [U^T, 0]] with U the correlation
   of the centred, sqrt(mass)-weighted coordinates; solvent atoms copied.
   out[nframes*3*natom] the fitted frames (the coordinates qcalc's later
   calculations of the frame see); status[nframes] 0, 1 (|det U| < 1e-9) or 2
   (det U < 0 with a degenerate pair), where the frame is only moved to the
   reference's centre of mass, as qcalc leaves it. */
int qgpu_calc_fit(const double *frames, int32_t nframes, int32_t natom, int32_t nsol, const int32_t *mask,
                  int32_t nmask, const double *mass, const double *xref, double *out, int32_t *status);
/* Centre of mass of the masked atoms (calc_com.f90 COM_calc); mass per atom
   (natom).  out[nframes*3]. */
int qgpu_calc_com(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                  const double *mass, double *out);
/* Kinetic energy of the centre of mass of a mask (calc_com_ke.f90
   COM_KE_calc) from consecutive frames frame_length fs apart: translational
   0.5 M |c_f - c_{f-1}|^2 / dt^2 and rotational sum over the principal axes j
   of the frame's inertia tensor of |L_j|^2 / (2 I_j), L_j the angular
   momentum of the atoms' positions relative to the centre, less their
   components along axis j, with velocities from the change of those relative
   positions; both times 2390 (the reference's integer conversion factor,
   g/mol A^2/fs^2 to kcal/mol).  Frame 0 is its own predecessor (zero).  mass
   per atom (natom).  out[2*nframes]: (translational, rotational) kcal/mol. */
int qgpu_calc_com_ke(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask, int32_t nmask,
                     const double *mass, double frame_length, double *out);
/* Geometry (calc_geom.f90 dist_calc / angle_calc / torsion_calc): measurement
   m uses kind[m] (2 distance, 3 angle, 4 torsion) atoms atoms[4*m ...].
   out[nframes*nmeas]: A, or degrees (torsions signed). */
int qgpu_calc_geom(const double *frames, int32_t nframes, int32_t natom, int32_t nmeas, const int32_t *atoms,
                   const int32_t *kind, double *out);
/* Radial distribution counts (calc_rdf.f90 RDF_calc): every pair of a mask-1
   atom and a different mask-2 atom, distance as the reference forms it in
   single precision (minimum image when box != NULL: boxlength[3]), bin
   int(dist/radius*nbins + 1) for dist < radius.  counts[nbins] summed over all
   frames; the normalisation of RDF_finalize (shell volume, frames, mask-1
   atoms) is the caller's.  nbins <= 8192, nframes <= 65535. */
int qgpu_calc_rdf(const double *frames, int32_t nframes, int32_t natom, const int32_t *mask1, int32_t n1,
                  const int32_t *mask2, int32_t n2, double radius, int32_t nbins, const double *box, int64_t *counts);
/* Nonbonded energies over pair lists (calc_nb.f90 nb_calc_lists; replaces
   the per-frame calls of qcalc.f90:745, nb_calc, and of nb_qp_calc, one list
   per residue): for each frame and list l the sums over its pairs p in
   [list_start[l], list_start[l+1]) (atoms pairs[2*p], pairs[2*p+1]) of
     Vlj += lambdas[s]*(AA*r^-12 - BB*r^-6)                      (arith 0)
     Vlj += lambdas[s]*(sqrt(BB)*AA^6*r^-6*(AA^6*r^-6 - 2))       (arith 1)
     Vel += lambdas[s]*qq/r
   over the states s < nstates, with the per-pair products AA, BB, qq stored
   pair-major ([p*nstates + s]; one state with lambdas {1} for the plain
   topology form).  A pair at r = 0 adds nothing.  The lists and their
   products are the caller's (nb_make_list, calc_nb.f90:334-759, built once
   before the frames).  list_start[nlist + 1], list_start[0] = 0.
   out[(f*nlist + l)*2 ..]: (Vlj, Vel), kcal/mol.  nframes <= 65535. */
int qgpu_calc_nb(const double *frames, int32_t nframes, int32_t natom, int32_t nlist, const int64_t *list_start,
                 const int32_t *pairs, int32_t nstates, const double *lambdas, const double *AA, const double *BB,
                 const double *qq, int32_t arith, double *out);

#ifdef __cplusplus
}
#endif
#endif /* QGPU_H */
