/*
 * ermod_gpu.h -- C ABI of the GB300 (sm_103a) energy-representation path.
 *
 * The entry points replace the body of ERmod's per-frame driver `engconst`
 * (engproc.F90:301-448) from the PME set-up (engproc.F90:355-383) through the
 * placement loop (engproc.F90:388-392: get_uv_energy + update_histogram).  A Fortran
 * host keeps enganal/setconf/insertion/engstore, the namelists and the output files,
 * and calls these functions through ISO_C_BINDING (include/ermod_gpu.f90).
 *
 * Conventions (those of the Fortran state in engmain.F90:252-301):
 *   - every array argument is caller-owned HOST memory unless the function name ends
 *     in `_device`; the library copies what it needs and owns its device memory;
 *   - arrays are column-major; index VALUES held in arrays are 1-based
 *     (mol_begin_index, ljtype, tagslt);
 *   - coordinates in Angstrom, energies in kcal/mol, charges already multiplied by
 *     18.22261721 (setconf.F90:829), temperature as kT in kcal/mol (setconf.F90:313);
 *   - every function returns an ermod_status (0 = success); nothing aborts or traps.
 * Threading: one context per host thread and device; a context is not reentrant.
 */
#ifndef ERMOD_GPU_H
#define ERMOD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2 added ermod_params.boxshp; a version-1 struct (without it) is still accepted and
 * means a periodic system. */
#define ERMOD_ABI_VERSION 2

/* Status codes.  The 1xx codes map one-to-one to ERmod's halt_with_error / warning
 * identities (mpiproc.F90:203-264) so that a Fortran wrapper can call
 * halt_with_error itself with the reference's message. */
typedef enum ermod_status {
  ERMOD_OK = 0,
  ERMOD_E_ENG_MIN = 101,   /* 'eng_min': energy at or below the first bin edge (engproc.F90:992-995) */
  ERMOD_E_ENG_SFT = 102,   /* 'eng_sft': solution-mode energy beyond the soft region (engproc.F90:999-1005) */
  ERMOD_E_ENG_BUG = 103,   /* 'eng_bug' (engproc.F90:975,986,997) */
  ERMOD_E_ENG_CNS = 104,   /* 'eng_cns': solvent with uvspec <= 0 (engproc.F90:817) */
  ERMOD_E_RCP_CNS = 105,   /* 'rcp_cns' (recpcal.F90:335,474) */
  ERMOD_E_RCP_FST = 106,   /* 'rcp_fst': the solute is a solvent (recpcal.F90:469) */
  ERMOD_E_INS_GEO = 107,   /* 'ins_geo': random or slab insertion in a non-periodic system (insertion.F90:155,186) */
  ERMOD_E_SET_PRS = 108,   /* 'set_prs': a non-periodic system needs NVT and bare Coulomb (setconf.F90:368-372) */
  ERMOD_E_ENG_SLB = 109,   /* 'eng_slb': slab configuration check in a non-periodic system (engproc.F90:1088) */
  ERMOD_W_MBIN = 110,      /* 'mbin' warning without force_calculation (engproc.F90:1010-1015) */
  ERMOD_E_INS_SIZ = 111,   /* 'ins_siz': solute structures of different sizes (insertion.F90:440,463-464) */
  ERMOD_E_PARAM = 120,     /* invalid argument or call order */
  ERMOD_E_NONCUBOID = 121, /* non-cuboid cell: the reference stops (realcal.F90:859-866) */
  ERMOD_E_UNSUPPORTED = 122, /* a mode the GPU path does not implement (cltype != PME) */
  ERMOD_E_CUDA = 130,      /* CUDA runtime error (see ermod_last_error_string) */
  ERMOD_E_CUFFT = 131,     /* cuFFT error */
  ERMOD_E_NOMEM = 132,     /* device allocation failed */
  ERMOD_E_DEVICE = 133     /* device-side check failed (index out of range) */
} ermod_status;

/* Arithmetic of the per-placement path. */
enum {
  ERMOD_PRECISION_FP64 = 0,  /* plain path: FP64 everywhere, spread + D2Z/Z2D, one placement at a time */
  ERMOD_PRECISION_MIXED = 1  /* batched path: FP32 grids and pair terms, FP64 totals and sums */
};

/* &ene_param subset that the path reads (engmain.F90:331-343, defaults setconf.F90:188-303). */
typedef struct ermod_params {
  int32_t abi_version;       /* ERMOD_ABI_VERSION */
  int32_t slttype;           /* 1 solution, 2 reference rigid, 3 reference flexible */
  int32_t estype;            /* 1 NVT, 2 NPT (volcorrect, engproc.F90:871-887) */
  int32_t cltype;            /* must be 2 (PME) */
  int32_t ljswitch;          /* 0 CHARMM pot, 1 GROMACS pot, 2 CHARMM force, 3 GROMACS force */
  int32_t splodr;            /* PME spline order (4, 6 or 8) */
  int32_t ms1max, ms2max, ms3max; /* PME grid */
  int32_t wgtslf;            /* weighting by the solute self energy */
  int32_t corrcal;           /* accumulate ecorr */
  int32_t selfcal;           /* accumulate eself */
  int32_t force_calculation; /* continue after the 'mbin' warning */
  int32_t precision;         /* ERMOD_PRECISION_* */
  int32_t batch;             /* placements per batch in the mixed path (0 = automatic) */
  int32_t count_mirror;      /* also keep an exact int64 unweighted ecorr count matrix */
  double elecut, lwljcut, upljcut, screen;
  double temp;               /* kT in kcal/mol */
  double block_threshold;    /* accepted for interface parity; the GPU path needs no cell list */
  int32_t boxshp;            /* 1 periodic, 0 non-periodic (bare Coulomb, NVT; engmain.F90:306) */
  int32_t finish_group;      /* mixed path: placements per molecule-energy block, 4 or 8 (0 = automatic;
                                the batch must be a multiple of it); a tile shape for autotuners */
} ermod_params;

typedef struct ermod_ctx ermod_ctx;

/* Fills p with the reference defaults for a PME run (setconf.F90:188-303). */
void ermod_default_params(ermod_params* p);

/* Context on CUDA device `device`.  Replaces recpcal_init's allocations
 * (recpcal.F90:42-85); the cuFFT plans are created here. */
int ermod_create(const ermod_params* p, int device, ermod_ctx** out);
int ermod_destroy(ermod_ctx* ctx);

/* Optional: order all work of this context on an existing cudaStream_t.  A placement call
 * forks from it onto the context's own streams (solute preparation, two batch streams,
 * the ordered accumulation and, with ecorr on, the flush) and joins them back into it
 * before it returns, so the caller sees one stream. */
int ermod_set_stream(ermod_ctx* ctx, void* cuda_stream);

/* Topology (engmain.F90:252-277).  mol_begin_index has nummol+1 entries (1-based),
 * sluvid/uvspec one per molecule, charge/ljtype one per site, ljene_mat and
 * ljlensq_mat are ljtype_max x ljtype_max column-major (setconf.F90:720-823). */
int ermod_set_topology(ermod_ctx* ctx, int nummol, int numatm, const int* mol_begin_index,
                       const int* sluvid, const int* uvspec, const double* charge,
                       const int* ljtype, int ljtype_max, const double* ljene_mat,
                       const double* ljlensq_mat);

/* Energy coordinate (engproc.F90:122-237, built by the host's enginit so that the
 * edges are the host's own): uvmax/uvsoft per solvent species, uvcrd(ermax),
 * escrd(esmax). */
int ermod_set_bins(ermod_ctx* ctx, int numslv, const int* uvmax, const int* uvsoft,
                   const double* uvcrd, int esmax, const double* escrd);

/* The host aggregate (hostspec; com_aggregate, insertion.F90:539-566): the molecules i
 * with host_mol[i] != 0 (0-based), and every site's mass sitemass[numatm] (engmain's
 * sitemass; center_of_mass weights, bestfit.F90:158-172).  Used by the configuration
 * check of insposition 2-4 and by device-generated placements with insorigin 2.  Call
 * after ermod_set_topology (which clears it).  A host without mass returns ERMOD_E_PARAM
 * ('bst_zrw' in the reference). */
int ermod_set_aggregate(ermod_ctx* ctx, const int* host_mol, const double* sitemass);

/* The reference structure (load_refstructure, insertion.F90:619-700): the refspec
 * molecules i with ref_mol[i] != 0, whose atoms in order have the reference coordinates
 * refhost_crd (3, n) and fitting weights refhost_weight (n), and the solute structure
 * refslt_crd (3, refslt_natom) with weights refslt_weight.  The weights are the host's
 * (read_refPDF_weight: 1 for heavy atoms, 0 for hydrogens and unlisted atoms).  Used by
 * the configuration check of insposition 5 and insstructure 1 (solution mode) and by
 * device-generated placements with insorigin 3 (reffit, insertion.F90:598-624).  Call
 * after ermod_set_topology (which clears it). */
int ermod_set_reference_structure(ermod_ctx* ctx, const int* ref_mol, const double* refhost_crd,
                                  const double* refhost_weight, int refslt_natom, const double* refslt_crd,
                                  const double* refslt_weight);

/* Solution-mode configuration check (check_mol_configuration, engproc.F90:1046-1100).
 * The reference skips a solution-mode placement whose solute fails it (get_uv_energy's
 * out_of_range, the loop's skipcond, engproc.F90:389-390).  Position (insposition):
 * 2 keeps a solute whose centre of mass lies at a distance in [lwreg, upreg] from that of
 * the host aggregate, 3 one whose offset from it along cell axis 3 does, 4 one whose
 * absolute offset does, 5 one whose RMSD from the reference solute structure, carried
 * into the frame by the best fit of the reference host onto the frame's host atoms, does;
 * 0, 1 and 6 test nothing (as in the reference).  Structure (insstructure 1): keeps a
 * solute whose best-fit RMSD from the reference solute structure lies in [lwstr, upstr].
 * A skipped placement adds nothing to any accumulator and leaves its uvengy and flceng
 * rows zero.  Slab checks (3, 4) of a non-periodic system return ERMOD_E_ENG_SLB; 2-4
 * need ermod_set_aggregate, 5 and insstructure 1 ermod_set_reference_structure with a
 * solute structure as long as every solute molecule ('eng_bug' otherwise: ERMOD_E_PARAM).
 * Call after ermod_set_topology (which switches the check off). */
int ermod_set_configuration_check(ermod_ctx* ctx, int insposition, double lwreg, double upreg, int insstructure,
                                  double lwstr, double upstr);

/* engconst prologue: cell inverse (engproc.F90:898-919), Green function when the
 * cell changed (recpcal.F90:111-152), solvent splines (recpcal.F90:328-340,408-442)
 * and the frame's solvent layout.  sitepos is (3, numatm), cell (3,3). */
int ermod_frame(ermod_ctx* ctx, const double* sitepos, const double* cell,
                double stat_weight_system);
int ermod_frame_device(ermod_ctx* ctx, const double* sitepos_device, const double* cell,
                       double stat_weight_system);

/* The placement loop (engproc.F90:388-392).  Placement p uses solute molecule
 * tagslt[p] (1-based).  solute_sitepos (3, nsite, nplace) holds the inserted solute's
 * coordinates (reference-solvent mode, insertion.F90:44-101) or is NULL (solution mode:
 * the frame's coordinates).  stat_weight_solute (nplace) may be NULL (all 1).
 * Optional outputs: uvengy_out (0:slvmax, nplace) -- the per-molecule energies of
 * get_uv_energy in tagpt order, uvengy(0) the solute self energy -- and
 * flceng_out (numslv, nplace).  Results accumulate into the context's
 * accumulators.  On an error status the accumulators keep the state of the last
 * complete batch and ermod_error_info tells which placement/molecule failed. */
int ermod_placements(ermod_ctx* ctx, int nplace, const int* tagslt, const double* solute_sitepos,
                     const double* stat_weight_solute, double* uvengy_out, double* flceng_out);
/* Same with tagslt/solute_sitepos/stat_weight_solute in device memory; the optional
 * outputs are device pointers too.  Returns without synchronising: the status of the
 * queued work is reported by the next ermod_sync.  Several calls may be queued between
 * two syncs: the first error among them is kept, and the calls after the failing one
 * accumulate nothing (the reference stops at its first error). */
int ermod_placements_device(ermod_ctx* ctx, int nplace, const int* tagslt_device,
                            const double* solute_sitepos_device,
                            const double* stat_weight_solute_device, double* uvengy_out_device,
                            double* flceng_out_device);
/* Waits for queued work, returns its status and starts a new sequence of calls. */
int ermod_sync(ermod_ctx* ctx);

/* engclear (engproc.F90:276-288). */
int ermod_clear(ermod_ctx* ctx);

/* Accumulators (engmain.F90:283-301), copied to host.  Any pointer may be NULL.
 * edens(ermax), ecorr(ermax,ermax) column-major, eself(esmax), slnuv(numslv),
 * minuv/maxuv(0:numslv), scalars[5] = {engnorm, engsmpl, avslf, voffset,
 * voffset_initialized}; ecorr_count(ermax,ermax) is the unweighted int64 mirror
 * sum_p insdst_p(i) insdst_p(j) (needs count_mirror). */
int ermod_get_accum(ermod_ctx* ctx, double* edens, double* ecorr, double* eself, double* slnuv,
                    double* minuv, double* maxuv, double* scalars, int64_t* ecorr_count);

/* Sizes known to the context: slvmax (physical molecules), ermax, esmax, numslv. */
int ermod_get_sizes(const ermod_ctx* ctx, int* slvmax, int* ermax, int* esmax, int* numslv);

/* Where the last error happened: placement index within the call, 1-based tagpt
 * position of the molecule (0 = the solute self energy) and its energy. */
int ermod_error_info(const ermod_ctx* ctx, int* placement, int* molecule, double* energy);

/* Per-phase device time (ms) accumulated since ermod_timing_reset with timing on;
 * names[i] are static strings.  Kernel launches issued by this library since the
 * last reset go to *launches. */
int ermod_timing_enable(ermod_ctx* ctx, int on);
int ermod_timing_reset(ermod_ctx* ctx);
int ermod_timing_get(ermod_ctx* ctx, int max_phases, double* ms, const char** names, int* nphases,
                     int64_t* launches);

/* Last CUDA/cuFFT error message of this thread. */
const char* ermod_last_error_string(void);
const char* ermod_status_string(int status);

/* ---- adjoint mode (mixed precision) --------------------------------------------------
 * Bin-resolved derivatives of the solute-solvent energy with respect to the solute's
 * per-site parameters.  For every placement of molecule solute_mol (1-based), every
 * solvent molecule k with energy u_k in bin iduv (getiduv, engproc.F90:927-1020) and
 * every solute site s:
 *   grad[p][iduv] += engnmfc * d u_k / d theta_p,   weight[iduv] += engnmfc
 * with theta_{3s} = q_s (charge in topology units, e x 18.22261721), theta_{3s+1} = LJ
 * epsilon of the site (ljene = sqrt(eps_s eps_t)), theta_{3s+2} = LJ sigma of the site
 * (ljlensq = ((sigma_s + sigma_t)/2)^2 for cmbrule 0, sigma_s sigma_t for cmbrule 1;
 * setconf.F90:779-823).  u_k is uvengy(k) of get_uv_energy (engproc.F90:662-756):
 * real-space LJ and erfc Coulomb, the PME reciprocal term and residual_ene.  The
 * conditional average <du/dtheta> in bin iduv is grad[p][iduv] / weight[iduv].
 * Per-molecule derivatives are FP32 and their sums FP64 in a fixed order.  Enable after
 * ermod_set_topology and ermod_set_bins (either one disables the mode again); ermod_clear
 * zeroes grad and weight; engstore-style merging treats them as it treats edens. */
int ermod_adjoint_enable(ermod_ctx* ctx, int solute_mol, int cmbrule);
/* grad: [3 nsite][ermax] (parameter-major), weight: [ermax]; *nparam = 3 nsite. */
int ermod_adjoint_get(ermod_ctx* ctx, double* grad, double* weight, int* nparam);

/* ---- several systems in one CUDA graph ------------------------------------------------
 * One step of nctx systems of uneven size (ermod_frame_device + ermod_placements_device
 * of each context: device coordinates sitepos_d[i], cell cells[9 i .. 9 i + 8], weight
 * stat_weight_system[i] (NULL: 1), nplace[i] placements of molecule solute_mol[i] with
 * device tags tag_d[i], solute coordinates sol_d[i] and weights sws_d[i] (NULL entries
 * allowed as in ermod_placements_device)) recorded once into a CUDA graph in which the
 * systems run concurrently, each with its own streams; ermod_graph_launch replays the
 * whole step as one launch.  This replaces, for a set of independent systems, the
 * per-system frame loop of enganal (enganal.F90:91-94) driving engconst.
 * Contract:
 *   - mixed precision only; every context has run one ordinary frame + placements step
 *     (its buffers and kernel attributes exist) and has no work queued;
 *   - the graph keeps device addresses and the host-side values given here (cells,
 *     counts, solute sizes); a launch reads whatever the device buffers hold, so new
 *     coordinates are written into the same buffers between launches; a new cell or
 *     count needs a new graph;
 *   - accumulators keep accumulating over launches (ermod_clear / ermod_get_accum as
 *     usual, between launches after ermod_graph_sync). */
typedef struct ermod_graph ermod_graph;
int ermod_graph_create(int nctx, ermod_ctx* const* ctx, const double* const* sitepos_d, const double* cells,
                       const double* stat_weight_system, const int* nplace, const int* solute_mol,
                       const int* const* tag_d, const double* const* sol_d, const double* const* sws_d,
                       ermod_graph** out);
/* Asynchronous on stream (a cudaStream_t; NULL: legacy default stream). */
int ermod_graph_launch(ermod_graph* g, void* stream);
/* Waits for the last launch; returns the first nonzero status of the systems in order
 * (as ermod_sync would for each; ermod_error_info on that context locates it). */
int ermod_graph_sync(ermod_graph* g);
int ermod_graph_destroy(ermod_graph* g);

/* ---- host-side set-up helpers (the reference's own set-up arithmetic) -------------- */

/* enginit's energy coordinate for one species (engproc.F90:163-218).
 * hist = {ecdmin, ecfmns, ecdcen, eccore, ecdmax, eclbin, ecfbin, ec0bin, finfac}.
 * ercrd must hold `large` doubles; writes ercrd[0..pemax-1]. */
int ermod_enginit_species(const double* hist, int pecore, int large, double* ercrd, int* pemax,
                          int* pesoft);
/* getscrn (setconf.F90:515-535): Ewald screening parameter from ewtoler. */
double ermod_getscrn(double ewtoler, double elecut, int distance_form);
/* LJ type table of setparam (setconf.F90:720-823).  nsite per-site (eps, len) pairs in
 * ljformat units -> ljtype(nsite) (1-based) and the ljtype_max x ljtype_max matrices
 * (column-major, capacity max_types^2). */
int ermod_lj_tables(int nsite, const double* eps, const double* len, int ljformat, int cmbrule,
                    int max_types, int* ljtype, int* ljtype_max, double* ljene_mat,
                    double* ljlensq_mat);
/* engstore's normalisation and rank merge (engproc.F90:475-560): merges nrank raw
 * accumulator sets (each as returned by ermod_get_accum) into rank 0's, including
 * the voffset max and exp rescale, then divides by engnorm.  Arrays are
 * [nrank][size] contiguous; ecorr may be NULL. */
int ermod_engstore_merge(int nrank, int slttype, int wgtslf, double temp, int ermax, int esmax,
                         int numslv, double* edens, double* ecorr, double* eself, double* slnuv,
                         double* minuv, double* maxuv, double* scalars);

/* ---- no counterpart in the reference ------------------------------------------------
 * ecorr(i, j) += weight[p] * hist[p][i] * hist[p][j] for p < nplace and, when
 * ecorr_count is not NULL, ecorr_count(i, j) += hist[p][i] * hist[p][j]: the ecorr update
 * of update_histogram (engproc.F90:841-853) for per-placement histograms (int32,
 * [nplace][ermax]) that the caller already holds.  hist, weight, ecorr (ermax x ermax,
 * symmetric) and ecorr_count are device pointers on the current device; stream is a
 * cudaStream_t (NULL: the legacy default stream).  Returns without synchronising.
 *
 * It allocates no device memory, for hosts that cannot let a library allocate inside
 * their step (a memory pool sized to the whole card; other streams that the implicit
 * device synchronisation of cudaFree would stall).  Its scratch is one fixed 8 MiB
 * device array, so nplace <= 4096, ermax <= 8192 and nplace * ermax <= 1048576, else
 * ERMOD_E_PARAM.  The first call on each device looks up that array's address: make it
 * before any stream capture.  The address is then kept for the life of the process, so
 * a host that resets the device (cudaDeviceReset) or tears down its primary context
 * must not call this entry point again afterwards.  All calls on a device share the
 * array, so calls that overlap on the GPU race. */
int ermod_ecorr_add_noalloc(const int* hist, const double* weight, int nplace, int ermax,
                            double* ecorr, int64_t* ecorr_count, void* stream);

/* ---- intermediate-state extension (extensions/Intermediate/engproc.F90) ---------------
 * Solution mode.  refs_density[ermax] is the reference-solvent distribution (engref's
 * third column, the largest over its .tt / .01-.99 files); its bins at or below 1e-30
 * form the zero-density set.  A placement none of whose occupied bins is in that set
 * belongs to the intermediate state: its engnmfc adds to soln_intm and norm_intm, its
 * histogram to edintm and its flceng to uvintm; every placement adds to soln_total
 * (the extension's update_histogram hunk).  ermod_clear zeroes edintm, uvintm and
 * norm_intm (its engclear hunk; soln_total and soln_intm run over the whole job). */
int ermod_intermediate_enable(ermod_ctx* ctx, const double* refs_density);
/* edintm[ermax], uvintm[numslv], totals[3] = {soln_total, soln_intm, norm_intm}. */
int ermod_intermediate_get(ermod_ctx* ctx, double* edintm, double* uvintm, double* totals);

/* ---- placements generated on the device (instslt, insertion.F90:76-99) --------------
 * insorigin 0: solute COM to the origin, 1 as given, 2 COM to the host aggregate's
 * (ermod_set_aggregate), 3 the best fit onto the reference solute structure carried into
 * the frame (reffit; ermod_set_reference_structure, insposition 5 or 6 only, as the
 * reference demands, and then a placement whose RMSD from that structure lies outside
 * [lwreg, upreg] is drawn again: check_solute_configuration, insertion.F90:569-595);
 * insposition 0 random in the cell,
 * 1 as given, 2 spherical shell lwreg..upreg, 3 slab in z, 4 symmetric slab, 5 random
 * translation within upreg + 3 x solute size, 6 uniform/Gaussian mixture with its
 * weight (engmain.F90:320-326, insertion.F90:133-316); insorient 0: random rotation
 * about the COM (rejection-sampled unit quaternion, q v q*), 1 none.  The random
 * stream is counter-based (Philox4x32-10): placement p uses counter offset + p under
 * key seed, so results do not depend on batching.  (The reference's Fortran
 * random_number stream is compiler specific and is not reproduced.) */
typedef struct ermod_insert_params {
  int32_t insposition, insorient, insorigin, pad_;
  double lwreg, upreg;
  uint64_t seed, offset;
} ermod_insert_params;
/* Writes nplace placements of an nsite solute (bfcoord (3, nsite) and mass host arrays,
 * the coordinates before insertion) into device sol_d (3, nsite, nplace) and, when not
 * NULL, their weights into device sws_d (1 except insposition 6).  Uses the cell of the
 * last ermod_frame*; asynchronous on the context's stream, ready for
 * ermod_placements_device. */
int ermod_generate_placements(ermod_ctx* ctx, int nplace, int nsite, const double* bfcoord, const double* mass,
                              const ermod_insert_params* ip, double* sol_d, double* sws_d);

/* ---- flexible solute (slttype 3: getsolute, insertion.F90:384-495) ------------------
 * The structures of SltConf in file order, conf (3, nsite, nconf) host array, and the
 * structure weights of SltWght's second column, weight[nweight] (nweight 0 or weight
 * NULL: every structure weighs 1).  insstructure 0 takes every structure; 1 only those
 * whose best-fit RMSD from the reference solute (rmsd_bestfit, bestfit.F90:245-252,
 * against ermod_set_reference_structure's refslt) lies in [lwstr, upstr].  Both files
 * wrap around on their own (setconf.F90:113-123 and insertion.F90:443-448), and a weight
 * is read with every structure, a rejected one included.  After this call
 * ermod_generate_placements ignores bfcoord (it may be NULL): placement g = offset + p
 * starts from the g-th accepted read of the wrapped file, i.e. read r = (g / na) nconf +
 * acc[g mod na] for the na accepted structures acc, with the initial weight
 * weight[r mod nweight] (then multiplied by insposition 6's factor), as instslt's
 * sequential reads give it; with insorigin 3 each placement fits its own structure onto
 * the reference solute carried into the frame.  nconf 0 removes the library.
 * ERMOD_E_INS_SIZ: nsite differs from the reference solute's (insstructure 1) or, later,
 * from ermod_generate_placements' nsite; ERMOD_E_PARAM when no structure is accepted
 * (the reference would read forever).  Synchronous. */
int ermod_set_solute_library(ermod_ctx* ctx, int nconf, int nsite, const double* conf, int nweight,
                             const double* weight, int insstructure, double lwstr, double upstr);

/* ---- engstore's output files (engproc.F90:594-657), for slvfe ------------------------
 * Written from merged, normalised accumulators (ermod_engstore_merge) in the
 * reference's layouts, with gfortran's edit conventions:
 *   engsln.xx / engref.xx  per bin '(g15.7,i5,g25.15)': repval('intn') energy
 *                          (engproc.F90:1185-1223), species, edens;
 *   slfeng.xx              per bin '(g15.7,g25.15)': repval('self'), eself;
 *   corsln.xx / corref.xx  one unformatted sequential record of ecorr(ermax, ermax)
 *                          (column major, little-endian 4-byte length markers);
 *   uvrange.tt             ' species     minimum        maximum' then '(i5,2f15.5)'
 *                          (or '(i5,f15.5,g18.5)' for maxuv >= 1e5) per species 0..numslv.
 * slvfe reads the text files list-directed and the record with one unformatted read
 * (slvfe.F90:466-488). */
int ermod_write_engdist(const char* path, int numslv, const int* uvmax, const int* uvsoft, const double* uvcrd,
                        const double* edens);
int ermod_write_selfdist(const char* path, int esmax, const double* escrd, const double* eself);
int ermod_write_corr(const char* path, int ermax, const double* ecorr);
int ermod_write_uvrange(const char* path, int numslv, const double* minuv, const double* maxuv);
/* The Gw.d field the writers use, into out (cap bytes, cap > w). */
int ermod_format_g(double x, int w, int d, char* out, int cap);

#ifdef __cplusplus
}
#endif
#endif /* ERMOD_GPU_H */
