/*
 * qnb.h -- C ABI of the GB300 (sm_103a) nonbonded engine for Q6's qdyn.
 *
 * The library replaces the bodies of qdyn's nonbonded routines for the
 * spherical boundary.  Every entry point below names the Q6 routine it
 * stands in for (paths relative to the Q6 source tree).  qdyn's MD loop,
 * topology, FEP and .inp files stay unchanged; its Fortran host calls these
 * functions through iso_c_binding.
 *
 * Conventions
 *  - All indices are 0-based (the Fortran shim subtracts 1 once, at create).
 *  - Coordinates x and the gradient d are natom x 3 doubles, atom-major
 *    (x0,y0,z0,x1,...), i.e. the memory layout of qdyn's TYPE(qr_vec) arrays.
 *  - d is the GRADIENT dU/dx (as in qdyn), and every call ADDS into d and into
 *    the energy records, it never overwrites them.
 *  - Multi-dimensional topology arrays use the Fortran (column-major) layout
 *    of the qdyn global they mirror; the offset formula is given per field.
 *  - Charges are the values qdyn holds after prep_sim, i.e. already scaled by
 *    sqrt(coulomb_constant) (Q6 src/simprep.f90:3714-3721).
 *  - Every function returns a qnb_status; 0 is success.  The library never
 *    falls back to a CPU path: without a usable CUDA device, qnb_create fails.
 *  - A context is used by one host thread at a time; all its work is issued on
 *    one CUDA stream owned by the context.
 */
#ifndef QNB_H
#define QNB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    QNB_OK = 0,
    QNB_ERR_ARG = 1,        /* invalid argument or topology                    */
    QNB_ERR_CUDA = 2,       /* CUDA runtime error (message: qnb_last_error)     */
    QNB_ERR_CAPACITY = 3,   /* a pair-list row overflowed; rebuilt lists larger */
    QNB_ERR_STATE = 4,      /* call out of order (e.g. energies before lists)   */
    QNB_ERR_NOMEM = 5,      /* device allocation failed                          */
    QNB_ERR_UNSUPPORTED = 6, /* topology feature outside this library's scope    */
    QNB_ERR_CONSTRAINT = 7  /* SHAKE did not converge in 1000 iterations          */
};

/* ---- precision forms ---------------------------------------------------- */
enum {
    QNB_PREC_FP64 = 0,  /* plain form: all arithmetic in FP64                     */
    QNB_PREC_MIXED = 1  /* FP32 pair math, 64-bit fixed-point forces/energies,
                           FP64 cut-off tests, LRF Taylor and energy reductions   */
};

/* ---- list kinds for qnb_export_pairs ------------------------------------ */
enum {
    QNB_LIST_PP = 0,   /* nbpp: solute-solute atom pairs (i, j)               */
    QNB_LIST_PW = 1,   /* nbpw: solute atom - solvent atom pairs (i, j)       */
    QNB_LIST_WW = 2,   /* nbww: solvent-solvent atom pairs (i, j)             */
    QNB_LIST_QP = 3,   /* nbqp: (Q index iq, solute atom j)                   */
    QNB_LIST_QW = 4,   /* nbqw: (Q index iq, solvent atom j)                  */
    QNB_LIST_PP14 = 5  /* subset of nbpp that are 1-4 pairs (LJ code 3)       */
};

/*
 * Static model description: a 0-based mirror of the qdyn module globals the
 * nonbonded path reads (Q6 src/globals.f90, src/topo.f90, src/qatom.f90).
 * The library copies everything at qnb_create and keeps no host pointer.
 */
typedef struct qnb_topology {
    int32_t natom;        /* nat_pro                                          */
    int32_t nat_solute;   /* solute atoms come first                          */
    int32_t nwat;         /* solvent molecules, solv_atom atoms each, after   */
    int32_t solv_atom;    /*   the solute                                     */
    int32_t solvent_type; /* 0 = SPC (Q6 SOLVENT_SPC), 1 = 3-atom, 2 = general */

    const double*  crg;   /* [natom] scaled charges                           */
    const int32_t* iac;   /* [natom] atom type, 0..natyps-1                   */
    const uint8_t* excl;  /* [natom] excluded (frozen/restrained) atoms       */
    const uint8_t* heavy; /* [natom] mass >= 4 (Q6 src/topo.f90:885-893)      */

    int32_t natyps;
    const double*  avdw;  /* [natyps*3], avdw[t*3+k] = iaclib(t+1)%avdw(k+1)  */
    const double*  bvdw;  /* [natyps*3], same layout                          */
    const uint8_t* ljcod; /* [natyps*natyps], ljcod[ti*natyps+tj] in {1,2}     */
    int32_t ivdw_rule;    /* 1 geometric, 2 arithmetic                        */
    double  el14_scale;

    int32_t ncgp;         /* charge groups: solute groups, then one per       */
    int32_t ncgp_solute;  /*   solvent molecule                               */
    const int32_t* cgp_first;   /* [ncgp] first slot in cgpatom               */
    const int32_t* cgp_last;    /* [ncgp] last slot in cgpatom (inclusive)    */
    const int32_t* cgp_iswitch; /* [ncgp] switch atom                         */
    const int32_t* cgpatom;     /* [cgp_last[ncgp-1]+1] atom indices          */
    int32_t iuse_switch_atom;   /* 1: group cut-off by switch atoms; 0: by
                                   any atom pair (nbpplis2/nbpwlis2/nbqplis2) */

    /* solute exclusions (listex + listexlong) and 1-4 pairs (list14 +
       list14long) as unordered atom pairs; order inside a pair is free       */
    int32_t nexcl_pairs;  const int32_t* excl_pairs;  /* [n*2] */
    int32_t n14_pairs;    const int32_t* pairs14;     /* [n*2] */

    /* Q atoms / FEP states (Q6 src/qatom.f90)                               */
    int32_t nqat, nstates;
    const int32_t* iqseq;     /* [nqat] atom index of each Q atom             */
    const double*  qcrg;      /* [nqat*nstates]  qcrg(iq,s) at iq + nqat*s     */
    const int32_t* qiac;      /* [nqat*nstates]  Q type, 0-based, same layout  */
    int32_t nqlib;            /* Q atom types                                 */
    const double*  qavdw;     /* [nqlib*3]  qavdw(t,k) at t*3 + k             */
    const double*  qbvdw;     /* [nqlib*3]                                    */
    int32_t qvdw_flag;        /* Q types redefined in the FEP file            */
    int32_t qq_use_library_charges;
    const double*  sc_lookup; /* [nqat*(natyps+nqat)*nstates]
                                 sc_lookup(iq,t,s) at iq + nqat*(t + (natyps+nqat)*s) */
    const int8_t*  qconn;     /* [nstates*nat_solute*nqat]
                                 qconn(s,i,iq) at s + nstates*(i + nat_solute*iq)       */
    int32_t nel_scale;        /* [el_scale] Q-Q electrostatic scaling          */
    const int32_t* el_scale_pairs; /* [n*2] Q indices                          */
    const double*  el_scale;       /* [n*nstates], pair p state s at p*nstates+s */
    int32_t nqexpnb;               /* [soft_pairs]                               */
    const int32_t* qexpnb_pairs;   /* [n*2] Q indices                            */

    double xpcent[3];   /* solute centre  (Q-atom list cut-off origin)        */
    double xwcent[3];   /* solvent centre (radial restraint origin)           */
    double rexcl_o;     /* exclusion radius                                   */
} qnb_topology;

typedef struct qnb_options {
    int32_t precision;   /* QNB_PREC_FP64 or QNB_PREC_MIXED                    */
    int32_t use_lrf;     /* [MD] lrf on/off                                    */
    int32_t device;      /* CUDA device ordinal                                */
    int32_t reserved;
} qnb_options;

/* NB_ENERGIES-like record for the classical terms (Q6 src/nrgy.f90:31-67). */
typedef struct qnb_energies {
    double pp_el, pp_vdw;  /* E%pp  */
    double pw_el, pw_vdw;  /* E%pw  */
    double ww_el, ww_vdw;  /* E%ww  */
    double lrf;            /* E%LRF */
} qnb_energies;

/* Per-state Q-atom record (part of OQ_ENERGIES, unweighted by lambda). */
typedef struct qnb_qenergies {
    double qq_el, qq_vdw;
    double qp_el, qp_vdw;
    double qw_el, qw_vdw;
} qnb_qenergies;

/* Spherical-boundary solvent restraint parameters (Q6 src/simprep.f90:4613-4891). */
typedef struct qnb_solvent_params {
    double fk_wsphere;   /* radial restraint force constant                    */
    double Dwmz, awmz;   /* Morse well depth / width                           */
    double rwat;         /* target solvent sphere radius                       */
    double boltz;        /* Boltzmann constant (kcal/mol/K)                    */
    int32_t wpol_restr;  /* polarisation restraint on/off                      */
    int32_t nwpolr_shell;/* shells (<= 16)                                     */
    double fkwpol;       /* polarisation force constant                        */
    double itdis;        /* pol_update interval in steps                       */
    double shell_rout[16], shell_dr[16], shell_cstb[16];
    double theta_corr[16]; /* initial theta_corr per shell (restart file)      */
} qnb_solvent_params;

typedef struct qnb_context qnb_context;

/* Last error message of the calling thread (static storage). */
const char* qnb_last_error(void);

/* Library/ABI version, e.g. 0x000300 for 0.3.0. */
int32_t qnb_version(void);

/* Copies the model, precomputes interaction tables (replaces
   precompute_interactions, src/simprep.f90:2860-2870, and the static Q lists
   make_nbqqlist/nbqqlist, src/nonbondene.f90:729-745, 3231-3282). */
int qnb_create(const qnb_topology* topo, const qnb_options* opt, qnb_context** out);

/* A context holding nwin lambda windows (or replicas) of the same topology,
   each with its own coordinates, lambdas, pair lists, LRF records and
   accumulators.  The *_dev entry points below process every window in the
   same kernel launches (grid.y = window).  The host-buffer entry points
   (qnb_make_pair_lists ... qnb_watpol) act on window 0, which is what one
   qdyn process per window uses.  No counterpart in the reference, which runs
   one process per window (tests/exclude_tests/inputs/excl/gen_inps.pl). */
int qnb_create_batch(const qnb_topology* topo, const qnb_options* opt, int32_t nwin, qnb_context** out);

/* Number of windows of the context. */
int qnb_window_count(qnb_context* ctx, int32_t* nwin);

/* Frees every device and host resource of the context. */
int qnb_destroy(qnb_context* ctx);

/* EQ(:)%lambda for the nstates FEP states (src/md.f90:974-1004), for every
   window of the context. */
int qnb_set_lambda(qnb_context* ctx, const double* lambda);

/* The same for window w only. */
int qnb_set_lambda_window(qnb_context* ctx, int32_t w, const double* lambda);

/* Replaces make_pair_lists(Rq,Rcq2,RcLRF2,Rcpp2,Rcpw2,Rcww2)
   (src/nonbondene.f90:749-837, spherical branch): group centres, pp/pw/ww
   lists with the LRF Taylor coefficients of groups beyond the cut-offs, and
   the qp/qw lists (kept after their first build when Rcq2 > rexcl_o^2). */
int qnb_make_pair_lists(qnb_context* ctx, const double* x, double Rq, double Rcq2,
                        double RcLRF2, double Rcpp2, double Rcpw2, double Rcww2);

/* Replaces pot_energy_nonbonds(E,EQ,md) (src/potene.f90:320-380, sphere
   branch): ww/qw (SPC fast path when geometric + SPC), pw, pp, qp and the LRF
   Taylor term.  With md == 0 only the qw and qp terms run, as in the
   reference.  EQ has nstates records. */
int qnb_pot_energy_nonbonds(qnb_context* ctx, const double* x, double* d,
                            qnb_energies* E, qnb_qenergies* EQ, int32_t md);

/* Replaces the calls nonbond_qq + nonbond_qqp (src/potene.f90:176-177). */
int qnb_nonbond_qq(qnb_context* ctx, const double* x, double* d, qnb_qenergies* EQ);

/* Solvent boundary set-up (wat_sphere / wat_shells results). */
int qnb_set_solvent_params(qnb_context* ctx, const qnb_solvent_params* p);

/* Replaces restrain_solvent (src/nonbondene.f90:6466-6544).  Tfree is the
   temperature of the free degrees of freedom from the integrator. */
int qnb_restrain_solvent(qnb_context* ctx, const double* x, double* d, double Tfree,
                         double* E_solvent_radial);

/* Replaces watpol(E,md) (src/nonbondene.f90:6548-6746) at MD step istep. */
int qnb_watpol(qnb_context* ctx, const double* x, double* d, int32_t istep, int32_t md,
               double* E_water_pol);

/* Current theta_corr, avtheta, avn_insh per shell (the restart-file state
   and the numbers watpol prints every itdis steps). */
int qnb_get_watpol_state(qnb_context* ctx, double* theta_corr, double* avtheta,
                         double* avn_insh);

/* ---- inspection (parity tests, diagnostics) ----------------------------- */

/* Number of atom pairs in list `kind` as the reference would hold them
   (nbpp_pair, nbpw_pair, nbww_pair, nbqp_pair, nbqw_pair). */
int qnb_list_size(qnb_context* ctx, int32_t kind, int64_t* n);

/* Writes the atom pairs of list `kind` (order unspecified) into i/j
   (capacity cap); *n receives the count.  QNB_ERR_CAPACITY if cap < count. */
int qnb_export_pairs(qnb_context* ctx, int32_t kind, int32_t* i, int32_t* j,
                     int64_t cap, int64_t* n);

/* Gather rows of the mixed form's last list build (QNB_PREC_MIXED only).
   Every listed solute group / water owns a row of partners, so each pair
   within a cut-off appears in the rows of both sides:
     QNB_ROWS_GP  solute group g -> solute atom j of a partner group (the
                  group itself included; Q atoms left out)
     QNB_ROWS_GW  solute group g -> water w     (nbpwlist selection)
     QNB_ROWS_WW  water w -> water v            (nbwwlist selection)
     QNB_ROWS_WG  water w -> solute group g     (nbpwlist selection)
   Writes window win's (row, partner) entries into row/partner (capacity
   cap); *n receives the count.  QNB_ERR_CAPACITY if cap < count.  Replaces
   no reference interface: it exposes the rows the selections of
   src/nonbondene.f90 (nbpplist 1777, nbpwlist 2842, nbwwlist 4274) are
   stored in here, so tests can compare them with those lists as sets. */
enum { QNB_ROWS_GP = 0, QNB_ROWS_GW = 1, QNB_ROWS_WW = 2, QNB_ROWS_WG = 3 };
int qnb_export_rows(qnb_context* ctx, int32_t win, int32_t kind, int32_t* row,
                    int32_t* partner, int64_t cap, int64_t* n);

/* LRF records as 43 doubles per charge group in the order of LRF_TYPE
   (src/globals.f90:503-509): cgp_cent(3), phi0, phi1(3), phi2(9), phi3(27). */
int qnb_get_lrf(qnb_context* ctx, double* lrf);

/* ---- device-resident interface (same work, inputs already in HBM) -------- */

/* Device buffers owned by the context: coordinates and gradient
   accumulators of all windows, nwin x natom x 3 doubles each, window-major.
   The *_dev entry points below read x from x_dev and add into d_dev without
   host copies. */
int qnb_device_buffers(qnb_context* ctx, double** x_dev, double** d_dev);

/* Copies host coordinates of all windows (nwin x natom x 3) into x_dev. */
int qnb_upload_coordinates(qnb_context* ctx, const double* x_all);

/* Copies the gradient accumulators of all windows into d_all (nwin x natom
   x 3); clears them on the device when clear != 0. */
int qnb_download_gradient(qnb_context* ctx, double* d_all, int32_t clear);

/* Stream the context issues its work on (cudaStream_t). */
int qnb_stream(qnb_context* ctx, void** stream);

int qnb_make_pair_lists_dev(qnb_context* ctx, double Rq, double Rcq2, double RcLRF2,
                            double Rcpp2, double Rcpw2, double Rcww2);

/* One full nonbonded evaluation of every window on device data:
   pot_energy_nonbonds(md=1), nonbond_qq/qqp, restrain_solvent and watpol.
   Energies are reduced on device; they are added to E[nwin], EQ[nwin*nstates]
   and Erst[nwin*2] (if non-NULL) only when sync != 0.
   Erst[2w] = solvent_radial, Erst[2w+1] = water_pol of window w. */
int qnb_compute_dev(qnb_context* ctx, double Tfree, int32_t istep, int32_t sync,
                    qnb_energies* E, qnb_qenergies* EQ, double* Erst);

/* nonbond_solvent_internal (src/nonbondene.f90:6082-6154): intra-molecular
   solvent pairs, replaces the nonbnd_solv_int list that
   prep_sim_precompute_solvent (src/simprep.f90:4003-4125) builds when the
   solvent has torsions.  ij[2k], ij[2k+1]: 0-based atom offsets inside a
   solvent molecule; A, B, el: the pair's vdWA, vdWB, elec.  Every molecule's
   pairs are evaluated in pot_energy_nonbonds (md) into E.ww.  n = 0 removes
   the list (the default). */
int qnb_set_solvent_internal(qnb_context* ctx, int32_t n, const int32_t* ij, const double* A, const double* B,
                             const double* el);

/* Launch-geometry autotuner (no counterpart in the reference).  Times, with
   CUDA events over `reps` evaluations of the current lists and coordinates
   (the evaluation's parallel branches off, so each class runs alone), the
   candidate blocks-per-SM of each per-step kernel class and of the list
   build, one parameter at a time, and keeps the fastest.  Results are
   independent of these choices.  The Q chunk (units per fixed-point
   conversion of the Q energies, default 8) is kept: it sets the grouping of
   FP32 partial sums, so changing it with qnb_set_tuning changes the Q
   energies at the FP32 rounding level (deterministically).  Needs built lists;
   restores the watpol running averages and clears the gradient
   accumulators.  values (may be NULL) receives the QNB_TUNE_COUNT choices:
   solute rows, water rows, qp, qw (blocks per SM), Q chunk (units), LRF
   Taylor, LRF accumulation, row build (blocks per SM). */
enum { QNB_TUNE_COUNT = 8 };
int qnb_autotune(qnb_context* ctx, int32_t reps, int32_t* values);
int qnb_get_tuning(qnb_context* ctx, int32_t* values);
int qnb_set_tuning(qnb_context* ctx, const int32_t* values);

/* The nonbonded side of one pot_energy call of a single-window context
   through host buffers, in one call: copies x (natom*3, the caller's memory)
   in, evaluates what qnb_compute_dev evaluates (pot_energy_nonbonds(md=1),
   nonbond_qq/qqp, restrain_solvent with Tfree and watpol at istep when
   solvent parameters are set, and any bonded / restraint / offdiag terms
   set on the context) as one graph replay, adds the gradient into d and the
   energies into E, EQ[nstates] and Erst[2] (solvent_radial, water_pol; each
   may be NULL).  One host synchronisation, where the separate entry points
   (qnb_pot_energy_nonbonds, qnb_nonbond_qq, qnb_restrain_solvent,
   qnb_watpol) take one each: src/potene.f90:140-170's nonbonded calls for a
   shim that makes them back to back on the same coordinates.  Needs the
   lists of a qnb_make_pair_lists* call; QNB_ERR_ARG for a batched context. */
int qnb_pot_energy_step(qnb_context* ctx, const double* x, double* d, double Tfree, int32_t istep,
                        qnb_energies* E, qnb_qenergies* EQ, double* Erst);

/* One step of every window of a (batched) context through host buffers, in
   one call with one host synchronisation: copies the coordinates of all
   windows (x_all, nwin x natom x 3; pinned memory makes the copy
   asynchronous) into HBM, rebuilds the pair lists with the cut-offs of the
   last qnb_make_pair_lists* call when rebuild_lists != 0 (qdyn's list update
   every NBcycle steps, src/md.f90:1661-1690, on this step's coordinates),
   evaluates what qnb_compute_dev evaluates, writes the gradient of all
   windows into d_all (nwin x natom x 3, overwritten; the device
   accumulators are cleared) and adds the energies into E[nwin],
   EQ[nwin*nstates] and Erst[nwin*2] (each may be NULL).  The same work as
   qnb_upload_coordinates + qnb_make_pair_lists_dev + qnb_compute_dev(sync)
   + qnb_download_gradient(clear), which wait on the device three or four
   times.  Needs lists built once (QNB_ERR_STATE otherwise). */
int qnb_step_host(qnb_context* ctx, const double* x_all, double* d_all, double Tfree, int32_t istep,
                  int32_t rebuild_lists, qnb_energies* E, qnb_qenergies* EQ, double* Erst);

/* Energies of the last qnb_compute_dev / qnb_group_compute evaluation of all
   windows, added into E[nwin], EQ[nwin*nstates], Erst[nwin*2] (waits for
   the context's stream). */
int qnb_get_energies_dev(qnb_context* ctx, qnb_energies* E, qnb_qenergies* EQ, double* Erst);

/* qnb_compute_dev replays its kernel sequence from a CUDA graph (default on;
   0 launches kernel by kernel).  A graph is captured on first use and again
   whenever list capacities, solvent parameters or Tfree change; the steps
   that update watpol's theta_corr use a second graph.  With qnb_profile on,
   the graph also records the per-class timing events; call
   qnb_profile_collect after each evaluation has finished (otherwise the
   next qnb_compute_dev waits for it before replaying). */
int qnb_set_graphs(qnb_context* ctx, int32_t enable);
int qnb_profile_collect(qnb_context* ctx);

/* Branches of the mixed form's evaluation (on by default): after the
   coordinate pack the solute rows run on the context's stream, the water
   rows and the step's further terms (qq, bonded, restraints, watpol) on a
   second stream, the Q-environment and LRF Taylor kernels on a third, all
   joined before the fixed-point gradient apply.  Every sum is fixed point,
   so results are the same with enable = 0, which runs them in one stream
   (each kernel then has the device to itself, e.g. for per-kernel timing). */
int qnb_set_concurrency(qnb_context* ctx, int32_t enable);

/* A group of contexts (systems of different sizes, e.g. replicas of uneven
   sphere radii, on one device) evaluated as ONE CUDA graph launch: each
   context's kernel sequence is an independent branch of the graph, so the
   systems run concurrently.  qnb_group_compute is qnb_compute_dev(sync = 0)
   for every member; read energies with qnb_get_energies_dev and gradients
   with qnb_download_gradient.  Members must outlive the group; profiling
   must be off.  No counterpart in the reference (one process per window). */
typedef struct qnb_group qnb_group;
int qnb_group_create(qnb_context** ctxs, int32_t n, qnb_group** group);
int qnb_group_compute(qnb_group* group, double Tfree, int32_t istep);
int qnb_group_destroy(qnb_group* group);

/* Adjoint of the Q-atom energies (no counterpart in the reference; for
   force-field and EVB parameter fitting).  For every window w, Q atom iq and
   state s, at the current device coordinates and lists:
     dq[w*nqat*nstates + iq + nqat*s] = dE_s/d qcrg(iq,s)   (scaled charge)
     dA[...]                          = dE_s/d qA(iq,s)
     dB[...]                          = dE_s/d qB(iq,s)
   E_s is the state's unweighted Q-atom nonbonded energy (qq + qp + qw).  qA,
   qB are the Q atom's code-1 LJ factors (qavdw(qiac(iq,s),1) with Q atom
   types, iaclib(iac)%avdw(1) otherwise), combined with the partner's as the
   topology's rule does (src/simprep.f90:3326-3341): geometric A_pair = qA a_j,
   B_pair = qB b_j; arithmetic A_pair = (qA + a_j)^12 qB b_j, B_pair =
   2 (qA + a_j)^6 qB b_j.  1-4 and soft pairs use other factors and do not
   contribute to dA/dB.  Each state's energy depends on that state's
   parameters only, so the gradient of the gap E2-E1 is dE2/dp(.,2) for the
   state-2 parameters and -dE1/dp(.,1) for the state-1 parameters.  Pair
   terms are recomputed from the lists with FP64 geometry in both precision
   forms; the sums use FP64 atomics (equal to rounding between calls). */
int qnb_q_adjoint_dev(qnb_context* ctx, double* dq, double* dA, double* dB);

/* Number of kernel launches the context issued since the last call. */
int qnb_take_launch_count(qnb_context* ctx, int64_t* n);

/* ---- event profiler (diagnostics; no counterpart in the reference) -------- */
/* Kernel classes, in the order qnb_kernel_times reports them. */
enum {
    QNB_K_WW = 0, QNB_K_QW, QNB_K_PW, QNB_K_PP, QNB_K_QP, QNB_K_LRF_TAYLOR, QNB_K_QQ,
    QNB_K_RESTRAIN, QNB_K_WATPOL, QNB_K_PACK, QNB_K_APPLY, QNB_K_BUILD, QNB_K_LRF_BUILD,
    QNB_K_BONDED, QNB_K_MD,
    QNB_K_COUNT
};

/* Brackets every launch of each kernel class with CUDA events on the
   context's stream while enable != 0. */
int qnb_profile(qnb_context* ctx, int32_t enable);
/* Profiling of the kernel classes whose bits (1 << QNB_K_*) are set only;
   0 turns profiling off.  Fewer events, less perturbation of the timing. */
int qnb_profile_classes(qnb_context* ctx, uint32_t mask);

/* Total milliseconds and launches per kernel class since the last call
   (n entries, n <= QNB_K_COUNT); resets the totals. */
int qnb_kernel_times(qnb_context* ctx, double* ms, int64_t* launches, int32_t n);

/* ---- bonded terms (FP64) -----------------------------------------------------
   pot_energy_bonds (src/potene.f90:258-317) and the Q-atom bonded terms of
   pot_energy (src/potene.f90:180-189), evaluated inside qnb_compute_dev and
   qnb_md_run once set:
     bond       0.5 fk (r - b0)^2                       src/bondene.f90:182-245
     angle      0.5 fk (theta - theta0)^2               src/bondene.f90:41-113
     Urey-Bradley (urey_bradley != 0) ureyfk (r13 - r0)^2 on the same angles
     torsion    fk (1 + cos(rmult phi - delta)) / paths src/bondene.f90:689-762
     improper   imp_type 1: 0.5 fk wrap(phi - phi0)^2;  src/bondene.f90:247-317
                imp_type 2: fk (1 + cos(2 phi - phi0))  src/bondene.f90:319-385
     Q bond     Dmz (e^2 - 2e) + 0.5 fk db^2, e = exp(-amz db)   src/bondene.f90:506-553
     Q angle / torsion / improper as above per state (Q torsions without the
     paths divisor), energies unweighted per state, gradient weighted by
     lambda_s                                           src/bondene.f90:387-448, 555-688
   Lists are 0-based atoms and library codes; a code < 0 skips the term (the
   topology entries qdyn removes: redefined in the FEP file, or constrained by
   SHAKE, src/simprep.f90:1050-1135, 2330-2345, 4395-4491).  Entries [0,
   n*_solute) count as solute (E%p), the rest as solvent (E%w).  Angles in
   radians; torsion libraries hold 1/paths.  Q terms hold one code per state
   (q*_code[term * nstates + s]).  Couplings of Q angles, torsions and
   impropers to Morse bonds are not supported. */
typedef struct qnb_bonded {
    int32_t nbonds, nbonds_solute;     const int32_t* bonds;      /* [3n] i j code    */
    int32_t nbondlib;                  const double* bondlib;     /* [2n] fk b0       */
    int32_t nangles, nangles_solute;   const int32_t* angles;     /* [4n] i j k code  */
    int32_t nanglib;                   const double* anglib;      /* [4n] fk theta0 ureyfk ureyr0 */
    int32_t ntors, ntors_solute;       const int32_t* torsions;   /* [5n] i j k l code */
    int32_t ntorlib;                   const double* torlib;      /* [4n] fk rmult delta 1/paths */
    int32_t nimps, nimps_solute;       const int32_t* impropers;  /* [5n] i j k l code */
    int32_t nimplib;                   const double* implib;      /* [2n] fk phi0     */
    int32_t imp_type;                  /* 1 harmonic, 2 periodic                   */
    int32_t urey_bradley;              /* CHARMM force fields: Urey-Bradley on     */
    int32_t nqbonds;    const int32_t* qbonds;    const int32_t* qbond_code;   /* [2n], [n*S] */
    int32_t nqbondlib;  const double* qbondlib;   /* [4n] Dmz amz r0 fk          */
    int32_t nqangles;   const int32_t* qangles;   const int32_t* qangle_code;  /* [3n], [n*S] */
    int32_t nqanglib;   const double* qanglib;    /* [4n] fk theta0 ureyfk ureyr0 */
    int32_t nqtors;     const int32_t* qtorsions; const int32_t* qtorsion_code; /* [4n], [n*S] */
    int32_t nqtorlib;   const double* qtorlib;    /* [3n] fk rmult delta         */
    int32_t nqimps;     const int32_t* qimpropers; const int32_t* qimproper_code; /* [4n], [n*S] */
    int32_t nqimplib;   const double* qimplib;    /* [2n] fk phi0                */
    /* [angle_couplings], [torsion_couplings], [improper_couplings]: rows
       (Q term, Q bond, 1 to couple to bond breaking) with 0-based indices
       into qangles / qtorsions / qimpropers and qbonds.  The term's energy
       and force are scaled by gamma = EMorseD of the bond (1 - EMorseD when
       breaking; 1 while the bond is shorter than r0), and the bond's atoms
       get dMorse * (unscaled term energy), as qangle, qurey_bradley,
       qtorsion and qimproper do (src/bondene.f90:387-688).  A coupled bond
       absent in a state (code -1) gives gamma 1 there. */
    int32_t nang_coupl; const int32_t* ang_coupl; /* [3n]                       */
    int32_t ntor_coupl; const int32_t* tor_coupl; /* [3n]                       */
    int32_t nimp_coupl; const int32_t* imp_coupl; /* [3n]                       */
} qnb_bonded;

/* Bonded energies of the last evaluation of every window: Eb[w*8 + k] =
   E%p%bond, angle, torsion, improper, E%w%bond, angle, torsion, improper;
   EQb[(w*nstates + s)*4 + k] = EQ(s)%q%bond, angle, torsion, improper. */
int qnb_set_bonded(qnb_context* ctx, const qnb_bonded* b);
int qnb_get_bonded_energies(qnb_context* ctx, double* Eb, double* EQb);

/* offdiag (src/nonbondene.f90:6238-6260): the EVB couplings of Q-state pairs
   (states[2k], states[2k+1], 0-based) as functions of the distance of two Q
   atoms (qatoms[2k], qatoms[2k+1], 0-based Q indices):
   Hij = A[k] exp(-mu[k] r_kl).  Evaluated inside qnb_compute_dev and every
   qnb_md_run step; n = 0 removes them.  qnb_get_offdiag returns the last
   evaluation's Hij and r_kl, [nwin][n] each (either may be NULL); these are
   the OFFD records put_ene writes. */
int qnb_set_offdiag(qnb_context* ctx, int32_t n, const int32_t* states, const int32_t* qatoms, const double* A,
                    const double* mu);
int qnb_get_offdiag(qnb_context* ctx, double* Hij, double* rkl);

/* Monitor groups, the [nonbonded_monitor] input section: nbmonitorlist +
   nonbond_monitor (src/nonbondene.f90:4517-4680).  ngroups atom groups of
   solute atoms (group g = atoms[group_first[g] .. group_first[g+1]), 0-based)
   and npairs pairs of them (pairs[2k], pairs[2k+1]).  Per pair and state the
   Coulomb and LJ energies of every interacting atom pair between the two
   groups, with the parameters the force loops use: Q-Q pairs the static
   Q-Q entry (soft pairs, soft-core), Q-P pairs the q-p or Q-bonded-P values,
   P-P pairs pp_precomp's (1-4 scaled, excluded pairs left out).  Evaluated
   inside qnb_compute_dev and every qnb_md_run step (FP64); npairs = 0
   removes them.  qnb_get_monitor_energies returns the last evaluation,
   out[((w*npairs + k)*nstates + s)*2 + {0: Vel, 1: Vlj}].  Two index slips
   of nbmonitorlist are not reproduced: its P-P branch indexes pp_map by the
   loop counters and its Q-P branch qp_precomp with the arguments swapped;
   both take the two atoms' own pair values here. */
int qnb_set_monitor_groups(qnb_context* ctx, int32_t ngroups, const int32_t* group_first, const int32_t* atoms,
                           int32_t npairs, const int32_t* pairs);
int qnb_get_monitor_energies(qnb_context* ctx, double* out);

/* Group contributions, the [group_contribution] input section: exc_assign +
   calculate_exc (src/simprep.f90:2879-2945, src/nonbondene.f90:6825-6920).
   mask[g*nat_solute + i] != 0 puts solute atom i in group g.  Per group and
   state the energies of the interactions calculate_exc subtracts from EQ:
   every Q-Q pair with an atom in the group, and every pair of a Q atom with
   a non-Q solute atom of the group (Q-bonded-P pairs included), at any
   distance.  out[((w*ngroups + g)*nstates + s)*4 + {0: qq el, 1: qq vdw,
   2: qp el, 3: qp vdw}]; the energy file's array of the group holds EQ minus
   these (el, vdw or both by the group's calculation type).  ngroups = 0
   removes them. */
int qnb_set_group_exclusions(qnb_context* ctx, int32_t ngroups, const uint8_t* mask);
int qnb_get_group_exclusions(qnb_context* ctx, double* out);

/* Periodic boundary conditions (use_PBC): a rectangular box of edges
   boxlength[3] (A) and the Q-list switching atom qswitch (0-based atom; the
   FEP file's [PBC] switching_atom).  From the next qnb_make_pair_lists* call
   the lists and energies follow the *_box routines: nbpplist_box,
   nbpwlist_box, nbwwlist_box (switch atoms / first solvent atoms within the
   cut-off in the minimum image, src/nonbondene.f90:1643-1775, 2730-2841,
   4174-4273), nbqplist_box / nbqwlist_box (groups with any atom, waters with
   the first atom, within Rcq of qswitch, 3747-3860, 3949-4026), and
   nonbond_pp_box, _pw_box, _ww(_spc)_box, _qp_box, _qw(_spc)_box
   (4763-6077), every pair at x_j + boxlength*nint((x_a - x_b)/boxlength) of
   its units' reference atoms.  The static Q-Q lists keep plain distances, as
   nonbond_qq does.  Cut-offs must not exceed half the shortest edge.
   With iuse_switch_atom = 0 the pp / pw lists are nbpplis2_box /
   nbpwlis2_box's (any atom pair inside).  With LRF on, unit pairs between
   the cut-off and RcLRF in the minimum image feed the LRF moments as in
   nbpplist_box_lrf / nbpwlist_box_lrf / nbwwlist_box_lrf (1910-2055,
   2957-3085, 4397-4515), each source at x_i - boxlength*nint((x_switch -
   centre)/boxlength) (lrf_update, 636-643), and lrf_taylor covers every
   non-Q atom.  Excluded atoms take part like any other atom (the box lists,
   lrf_taylor and temperature() test no exclusion under use_PBC); solvent
   internal pairs use the minimum image (nonbond_solvent_internal_box,
   6158-6228).  boxlength = NULL returns to the sphere (and its exclusions).
   With iuse_switch_atom = 0 and LRF on, a unit pair with a solute group
   feeds the LRF moments when none of its minimum-image atom pairs (a water
   by its first atom) lies within the cut-off and one lies within RcLRF
   (nbpplis2_box_lrf / nbpwlis2_box_lrf, 1220-1367, 2359-2491; FP64 terms in
   both precision forms).  Not supported with a box (QNB_ERR_UNSUPPORTED):
   solvent restraints.  Constant pressure is the caller's; put_back_in_box:
   qnb_set_put_back_in_box. */
int qnb_set_box(qnb_context* ctx, const double* boxlength, int32_t qswitch);

/* fix_shell (src/potene.f90:386-423), evaluated inside qnb_compute_dev and
   qnb_md_run once set: excluded atoms (the topology's excl flags) with
   fk_fix and shell atoms (shell[i] != 0, as make_shell / make_shell2 mark
   them, src/topo.f90:1426-1491) with fk_pshell are restrained harmonically
   to xtop (natom x 3): E = 0.5 fk |x - xtop|^2 into E%restraint%fix / %shell.
   xtop = NULL removes the restraint.  The freeze option: qnb_set_freeze. */
int qnb_set_shell_restraint(qnb_context* ctx, const double* xtop, const uint8_t* shell, double fk_fix,
                            double fk_pshell);
/* excluded_freeze (src/potene.f90:401-405, src/bondene.f90:791-855): with
   freeze != 0 every evaluation puts the excluded atoms back to xtop with zero
   velocity (the MD velocities, once qnb_md_init ran) and zero fix_shell force
   constant, and the restraint sections skip excluded atoms in their
   `ih = 1` (all-atom) selections.  Needs qnb_set_shell_restraint's xtop. */
int qnb_set_freeze(qnb_context* ctx, int32_t freeze);
/* The input file's restraint sections, p_restrain (src/bondene.f90:764-1020),
   evaluated inside qnb_compute_dev and qnb_md_run once set (FP64):
     sequence  atoms seq_ij[2k]..seq_ij[2k+1] (heavy atoms, or all with
               seq_ih[k] = 1) restrained to xtop with seq_fk[k]: each atom
               (mode 0), their geometric centre (1; the reference's force on
               each atom is dr fk m_i / 12.010) or mass centre (2) -> E%restraint%protein
     position  atom pos_i[k] to pos_x[3k..] with per-axis pos_fk[3k..]
     distance  atoms dist_ij[2k], [2k+1], flat bottom between dist_d[2k] and
               dist_d[2k+1] (A), dist_fk[k]
     angle     atoms ang_ijk[3k..] at ang_theta[k] (degrees), ang_fk[k]
     wall      atoms wall_ij[2k]..[2k+1] (heavy, or all with wall_ih[k] = 1):
               half-harmonic beyond wall_d[k] from xwcent (fk wall_fk[k]),
               Morse inside (wall_aMorse, wall_dMorse) -> E%restraint%protein
   State-dependent kinds (position, distance, angle) carry *_state[k]: -1 for
   every state (the reference's 0: the energy goes to every state's
   EQ(s)%restraint, the force is unweighted), else the 0-based state s whose
   EQ(s)%restraint gets the energy and whose lambda weights the force.
   Atom indices 0-based; xtop is natom x 3.  r = NULL removes the restraints.
   With qnb_set_freeze on, excluded atoms leave the ih = 1 selections. */
typedef struct qnb_restraints {
    int32_t nseq;  const int32_t* seq_ij;  const double* seq_fk;  const int32_t* seq_ih;  const int32_t* seq_mode;
    int32_t npos;  const int32_t* pos_i;   const int32_t* pos_state; const double* pos_x;  const double* pos_fk;
    int32_t ndist; const int32_t* dist_ij; const int32_t* dist_state; const double* dist_d; const double* dist_fk;
    int32_t nang;  const int32_t* ang_ijk; const int32_t* ang_state; const double* ang_theta; const double* ang_fk;
    int32_t nwall; const int32_t* wall_ij; const double* wall_d;   const double* wall_fk;
    const double* wall_aMorse; const double* wall_dMorse; const int32_t* wall_ih;
} qnb_restraints;
int qnb_set_restraints(qnb_context* ctx, const qnb_restraints* r, const double* xtop);

/* Restraint energies of the last evaluation:
   Er[w*(5 + nstates) + k] = fix, shell, solvent_radial, water_pol, protein,
   then EQ(s)%restraint for every state s. */
int qnb_get_restraint_energies(qnb_context* ctx, double* Er);

/* ---- device-resident MD step (FP64) ----------------------------------------
   qdyn's leap-frog step for the spherical boundary with the Berendsen
   thermostat (md_run, src/md.f90:1687-1812), every window of the context on
   the device, no host round trip per step:
     every nbcycle steps  make_pair_lists (qnb_make_pair_lists_dev);
     pot_energy           d = 0, then the evaluation of qnb_compute_dev, with
                          restrain_solvent's Tfree taken on the device from the
                          window's last temperature() (src/md.f90:1379-1447);
     newvel_ber           per temperature group g (src/md.f90:1451-1466):
                          v = (v - d winv dt) sfact_g, xx = x, x = x + v dt;
     constraint           SHAKE (src/bondene.f90:1069-1150), then
                          v = (x - xx) / dt for every atom;
     temperature          Ekin, Temp, Tfree and the Berendsen factors
                          sfact_g = sqrt(1 + dt/tau_T (Temp0/Tfree_g - 1)).
   The step's forces are those of qnb_compute_dev: nonbonded, Q-Q, solvent
   boundary and, once qnb_set_bonded was called, the bonded terms.  Units as qdyn: masses in amu, time in fs (converted with qdyn's
   0.020462 per fs, src/md.f90:207 and 231), velocities in A per internal
   time unit. */
enum { QNB_MAX_TGROUPS = 4 };
typedef struct qnb_md_params {
    double stepsize;          /* time step (fs)                                  */
    double temp0;             /* Berendsen target temperature (K)               */
    double tau_t;             /* bath_coupling relaxation time (fs)             */
    double ndegf, ndegfree;   /* degrees of freedom: all atoms and non-excluded
                                 atoms (src/simprep.f90:2439-2440)              */
    int32_t ntgroups;         /* temperature coupling groups, 1..QNB_MAX_TGROUPS */
    int32_t nbcycle;          /* pair-list update interval (steps)              */
    int32_t tg_first[QNB_MAX_TGROUPS], tg_last[QNB_MAX_TGROUPS];   /* 0-based,
                                 inclusive atom range of each group             */
    double tg_ndegf[QNB_MAX_TGROUPS], tg_ndegfree[QNB_MAX_TGROUPS];
    double rq, rcq, rclrf, rcpp, rcpw, rcww;   /* cut-offs of the rebuilds (A)   */
} qnb_md_params;

/* Per window and step of qnb_md_run: the step's energies (as qnb_compute_dev
   reports them) and, after the step's temperature(), Ekin (E%kinetic), Temp,
   Tfree and the SHAKE iterations summed over the constrained molecules. */
typedef struct qnb_md_record {
    qnb_energies E;
    double solvent_radial, water_pol;
    double ekin, temp, tfree, shake_iterations;
    double fix, shell;        /* E%restraint%fix, %shell (qnb_set_shell_restraint) */
    double protein;           /* E%restraint%protein (qnb_set_restraints)          */
} qnb_md_record;

/* mass[natom] (amu); the constraints of molecule m are
   con_ij[2k], con_ij[2k+1] (0-based atoms) at distance con_dist[k] (A) for
   k in [mol_first[m], mol_first[m+1]), m < nmol.  Velocities start at 0. */
int qnb_md_init(qnb_context* ctx, const qnb_md_params* p, const double* mass, int32_t nmol,
                const int32_t* mol_first, const int32_t* con_ij, const double* con_dist);
/* Thermostat and integrator (the input's thermostat / integrator keys,
   src/md.f90:244-301), after qnb_md_init: thermostat 0 Berendsen (default),
   1 Nose-Hoover (nh_prop + newvel_nos, src/simprep.f90:2509-2550,
   src/md.f90:1505-1521; nhchains 2..10, nhq <= 0 for the default
   kbT/tau_T^2, the chain started as init_constraints does); integrator 0
   leap-frog (default), 1 velocity Verlet (half-step force updates before and
   after the move, as newvel_* do).  Langevin: qnb_md_set_langevin. */
int qnb_md_set_thermostat(qnb_context* ctx, int32_t thermostat, int32_t integrator, int32_t nhchains, double nhq);
/* Langevin thermostat (newvel_lan with uniform random forces, the
   default of src/md.f90:1468-1503, 1632-1648): friction <= 0 for 1/tau_T,
   integrator as qnb_md_set_thermostat.  The random forces are uniform draws
   from SplitMix64 keyed by (seed, window, step, atom component), not qdyn's
   randm sequence: the same distribution, not the same numbers. */
int qnb_md_set_langevin(qnb_context* ctx, int32_t integrator, double friction, uint64_t seed);
/* put_back_in_box (src/simprep.f90:4177-4352) for a periodic box, after
   qnb_md_init: molecule q is atoms[mol_first[q] .. mol_first[q+1]), the
   first nmol_solute of them solute; put_solute / put_solvent select which
   are wrapped (put_solute_back_in_box / put_solvent_back_in_box).  The box
   centre is boxcentre (rigid_box_centre), or NULL for the mean of the solute
   atoms (of all atoms without solute) at each call.  A molecule whose mass
   centre lies beyond half a box edge from the centre moves by one edge on
   that axis.  qnb_md_run calls it every NBcycle steps before the lists, as
   md_run does; qnb_put_back_in_box calls it now and returns the centres
   ([nwin][3], or NULL). */
int qnb_set_put_back_in_box(qnb_context* ctx, int32_t nmol, const int32_t* mol_first, const int32_t* atoms,
                            int32_t nmol_solute, int32_t put_solute, int32_t put_solvent, const double* boxcentre);
int qnb_put_back_in_box(qnb_context* ctx, double* boxcentre);
int qnb_md_set_velocities(qnb_context* ctx, int32_t window, const double* v);
/* x and/or v (natom x 3, either may be NULL) of one window. */
int qnb_md_get_state(qnb_context* ctx, int32_t window, double* x, double* v);
/* qdyn's start of dynamics on every window's device coordinates and
   velocities: initial_constraint (src/bondene.f90:1025-1048), then, if
   stop_cm != 0, stop_cm_translation (src/simprep.f90:4496-4518), then
   temperature() for Tfree and the thermostat factors of the first step.
   Required after qnb_md_init and after every qnb_md_set_velocities or
   coordinate upload before qnb_md_run. */
int qnb_md_prepare(qnb_context* ctx, int32_t stop_cm);
/* Qmin's steepest descent (src/minim.f90:891-935, 938-1160) on every
   window's device coordinates: nsteps steps of pot_energy (Tfree 0), then
   x -= d * scale with scale reset to initial_step whenever the largest atomic
   force rose above the previous step's and grown by 1.2 otherwise; SHAKE
   against the positions before the move; a window whose largest force is
   below force_cutoff stops moving.  max_move > 0 (an addition to Qmin's
   method, 0 = off) caps the largest atomic move of a step at max_move A,
   for strained starting structures whose first moves would break SHAKE.
   maxf (may be NULL) receives each window's largest force at the last step.
   Lists are rebuilt every nbcycle steps.  Velocities are untouched; call
   qnb_md_prepare before qnb_md_run. */
int qnb_md_minimize(qnb_context* ctx, int32_t nsteps, double initial_step, double force_cutoff, double max_move,
                    double* maxf);
/* nsteps steps of every window starting at step number istep0 (lists are
   rebuilt where istep % nbcycle == 0, watpol updates by istep).  rec (may be
   NULL): [nsteps][nwin] records; EQ (may be NULL): [nsteps][nwin][nstates];
   Eb (may be NULL): [nsteps][nwin][8 + 4*nstates], the bonded energies as
   qnb_get_bonded_energies orders them (classical, then Q per state).
   QNB_ERR_CONSTRAINT if SHAKE failed in any window (the coordinates are then
   those of the failed step). */
int qnb_md_run(qnb_context* ctx, int32_t nsteps, int32_t istep0, qnb_md_record* rec, qnb_qenergies* EQ,
               double* Eb);

/* ---- allocation-free entry point (no counterpart in the reference) ------- */

/* Water-water SPC energies and gradient without any device allocation, for
   callers that may not call cudaMalloc: a program held to a fixed device-memory
   budget by its scheduler or host application, a process whose own pool
   allocator already holds the device's free memory, or a timed step loop in
   which cudaMalloc/cudaFree would synchronise the device.  It is the FP64
   nbwwlist + nonbond_ww_spc
   computation: water pairs whose O atoms lie within rc2 (neither O excluded)
   each contribute LJ + Coulomb for O-O and Coulomb for the other eight atom
   pairs.
   Inputs and outputs are the caller's device buffers:
     x_dev    natom x 3 coordinates; waters are 3 atoms each, starting at
              atom first_water_atom (O, H, H);
     excl_dev optional excluded-atom flags (u8 per atom), or NULL;
     q_oxygen, q_hydrogen  scaled charges; A_oo, B_oo the O-O LJ A and B;
     d_dev    gradient, natom x 3, ADDED into;
     e_dev    2 doubles, el and vdW, ADDED into;
     stream   a cudaStream_t, or NULL for the legacy default stream.
   Scratch: a file-scope device array that holds 1,048,576 water pairs
   (8 MiB). Every GPU that loads the library keeps it until the process
   exits. More than 65,536 waters, or more pairs within the cut-off than the
   array holds, returns QNB_ERR_CAPACITY (message in qnb_last_error).  All
   calls on a device share the array: each call clears its counter first,
   and calls that overlap on the GPU (different streams or threads) race.
   The first call on a device looks up the array's device address
   (cudaGetSymbolAddress) with that device current.  The address is kept for the life of the
   process, so the entry point is not for use after a cudaDeviceReset.  The
   call waits on `stream` once, after the pair selection, to check the pair
   count.  The gradient and energies are added with FP64 atomics: repeated
   calls agree to rounding, not bit for bit. */
int qnb_ww_spc_noalloc(const double* x_dev, const uint8_t* excl_dev, int32_t first_water_atom, int32_t nwat,
                       double q_oxygen, double q_hydrogen, double A_oo, double B_oo, double rc2,
                       double* d_dev, double* e_dev, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QNB_H */
