/*
 * ermod_oracle.h -- FP64 CPU restatement of ERmod's per-frame energy-representation
 * path, used ONLY as test infrastructure (the checker for the CUDA path and the timed
 * CPU baseline).  Nothing in the product links, imports or calls this library.
 *
 * Parity status: partially pinned.  The reference (Fortran 90 + FFTW/MKL + LAPACK)
 * cannot be compiled in this environment (no Fortran compiler, no FFTW/MKL/LAPACK),
 * so this oracle is a line-by-line restatement of the reference routines, pinned by
 *   - the reference's only golden vectors (spline_test.F90:19-40, cardinal B-spline
 *     values of order 2 and 6),
 *   - analytic checks written for this project (PME vs a direct Ewald sum, the
 *     FFT vs numpy, LJ switch continuity, the default energy-coordinate edges,
 *     the histogram-normalisation invariant of slvfe.F90:495-512).
 *
 * Conventions follow the reference's Fortran state (engmain.F90:252-301):
 * arrays are column-major, index VALUES stored in arrays are 1-based
 * (mol_begin_index, ljtype, tagslt), coordinates are Angstrom, energies kcal/mol,
 * charges already scaled by 18.22261721 (setconf.F90:829).
 */
#ifndef ERMOD_ORACLE_H
#define ERMOD_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: same identities and values as the product's C-ABI. */
enum {
  ORC_OK = 0,
  ORC_E_ENG_MIN = 101, /* energy at or below the first bin edge (engproc.F90:992-995) */
  ORC_E_ENG_SFT = 102, /* SOLN energy beyond the soft region (engproc.F90:999-1005) */
  ORC_E_ENG_BUG = 103, /* engproc.F90:975,986,997 */
  ORC_E_ENG_CNS = 104, /* uvspec <= 0 for a solvent (engproc.F90:817) */
  ORC_E_RCP_CNS = 105, /* recpcal.F90:335,474 */
  ORC_E_RCP_FST = 106, /* solute listed as solvent (recpcal.F90:469) */
  ORC_E_SET_PRS = 108, /* non-periodic with NPT or a non-bare Coulomb (setconf.F90:368-372) */
  ORC_E_ENG_SLB = 109, /* slab configuration check of a non-periodic system (engproc.F90:1087) */
  ORC_W_MBIN = 110,    /* last-bin warning without force_calculation (engproc.F90:1010-1015) */
  ORC_E_PARAM = 120,   /* invalid argument */
  ORC_E_NONCUBOID = 121 /* realcal.F90:859-866 */
};

typedef struct orc_params {
  int32_t slttype;  /* 1 soln, 2 refs rigid, 3 refs flexible (engmain.F90:318) */
  int32_t estype;   /* 1 NVT, 2 NPT */
  int32_t ljswitch; /* 0..3 (engmain.F90:314) */
  int32_t splodr;
  int32_t ms1max, ms2max, ms3max;
  int32_t wgtslf, corrcal, selfcal, force_calculation;
  int32_t elmode;   /* 0: PME (cltype 2), 1: PPPM (cltype 3, recpcal.F90:205-319), 2: bare Coulomb (cltype 0) */
  double elecut, lwljcut, upljcut, screen;
  double temp;            /* kT in kcal/mol (setconf.F90:313) */
  double block_threshold; /* realcal cell size (setconf.F90:219) */
  int32_t boxshp;         /* 1 periodic, 0 non-periodic (engmain.F90:306) */
  int32_t reserved_;
} orc_params;

typedef struct orc_ctx orc_ctx;

/* --- single routines (unit-test hooks) --------------------------------------- */
/* spline.F90:26-59 */
double orc_spline_value(int order, double x);
/* setconf.F90:515-535 (scrtype 'dis' when dis != 0) */
double orc_getscrn(double ewtoler, double elecut, int dis);
/* engproc.F90:122-237 for one species.  hist = {ecdmin, ecfmns, ecdcen, eccore, ecdmax,
 * eclbin, ecfbin, ec0bin, finfac}; pecore as in &hist.  Writes ercrd[0..pemax-1]. */
int orc_enginit_species(const double* hist, int pecore, int large, double* ercrd, int* pemax,
                        int* pesoft);
/* 3-D real FFT with the reference's conventions (fft_iface.F90): forward
 * e^{-2 pi i}, backward e^{+2 pi i}, unnormalised, half-complex along axis 1.
 * real[K3][K2][K1] <-> cplx[K3][K2][K1/2+1] (interleaved re,im). */
int orc_fft_r2c_3d(int k1, int k2, int k3, const double* in, double* out);
int orc_fft_c2r_3d(int k1, int k2, int k3, const double* in, double* out);
/* LJ + screened-Coulomb pair energy of one site pair at squared distance dist,
 * as get_pair_energy_block computes it (realcal.F90:585-784). */
double orc_pair_energy(const orc_params* p, double ljeps, double ljsgm2, double qq, double dist2);

/* --- the per-frame path --------------------------------------------------------- */
int orc_create(const orc_params* p, orc_ctx** out);
void orc_destroy(orc_ctx* c);
/* mol_begin_index has nummol+1 entries (1-based). ljene_mat/ljlensq_mat are
 * ljtype_max x ljtype_max column-major. */
int orc_set_topology(orc_ctx* c, int nummol, int numatm, const int* mol_begin_index,
                     const int* sluvid, const int* uvspec, const double* charge,
                     const int* ljtype, int ljtype_max, const double* ljene_mat,
                     const double* ljlensq_mat);
int orc_set_bins(orc_ctx* c, int numslv, const int* uvmax, const int* uvsoft, const double* uvcrd,
                 int esmax, const double* escrd);
/* engconst prologue (engproc.F90:355-383): cell inverse, PME set-up, solvent splines. */
int orc_frame(orc_ctx* c, const double* sitepos, const double* cell, double stat_weight_system);
/* The placement loop (engproc.F90:388-392).  tagslt[p] is the 1-based solute molecule
 * of placement p; solute_sitepos (3, nsite, nplace) replaces the solute's frame
 * coordinates (REFS insertion) or is NULL (SOLN: frame coordinates are used).
 * uvengy_out (0:slvmax, nplace) and flceng_out (numslv, nplace) are optional.
 * nthreads <= 0 uses the OpenMP default. */
int orc_placements(orc_ctx* c, int nplace, const int* tagslt, const double* solute_sitepos,
                   const double* stat_weight_solute, double* uvengy_out, double* flceng_out,
                   int nthreads);
int orc_slvmax(const orc_ctx* c);
/* The host aggregate (hostspec; host_mol[i] != 0 for 0-based molecules) and sitemass. */
int orc_set_aggregate(orc_ctx* c, const int* host_mol, const double* sitemass);
/* The reference structure (load_refstructure, insertion.F90:619-700): refspec molecules
 * (ref_mol[i] != 0) with refhost_crd (3, n) and refhost_weight (n); the solute's
 * refslt_crd (3, refslt_natom) and refslt_weight. */
int orc_set_reference_structure(orc_ctx* c, const int* ref_mol, const double* refhost_crd,
                                const double* refhost_weight, int refslt_natom, const double* refslt_crd,
                                const double* refslt_weight);
/* check_mol_configuration (engproc.F90:1046-1100), solution mode: insposition 2 (sphere),
 * 3 (slab), 4 (symmetric slab) about the host aggregate, 5 (RMSD from the reference solute
 * carried into the frame by the host fit); insstructure 1 (best-fit RMSD in [lwstr, upstr]).
 * Rejected placements are skipped (engproc.F90:389-390), their uvengy/flceng rows zero. */
int orc_set_configuration_check(orc_ctx* c, int insposition, double lwreg, double upreg, int insstructure,
                                double lwstr, double upstr);
/* bestfit.F90 fit_a_rotate_b (:215-242): a (3, na) fitted onto refa (weights massa), the same
 * transform applied to b (3, nb) -> bout. */
int orc_fit_a_rotate_b(int na, const double* refa, const double* a, const double* massa, int nb,
                       const double* b, double* bout);
/* raw accumulators, engclear (engproc.F90:276-288) */
int orc_clear(orc_ctx* c);
/* scalars = {engnorm, engsmpl, avslf, voffset, voffset_initialized}; any pointer may be NULL */
int orc_get_accum(const orc_ctx* c, double* edens, double* ecorr, double* eself, double* slnuv,
                  double* minuv, double* maxuv, double* scalars);
/* PME reciprocal potential of the last placement processed with nthreads == 1
 * (cnvslt, real[K3][K2][K1]) and its self energy; for cross-checks. */
int orc_last_cnvslt(const orc_ctx* c, double* out, double* self_energy);
/* PME reciprocal energies alone: recpcal_prepare_solute + recpcal_energy for every
 * physical molecule (0 for the solute itself), plus the solute's reciprocal self energy. */
/* Per-molecule derivatives of uvengy(k) with respect to the solute's per-site charge,
 * LJ epsilon and LJ sigma (cmbrule 0 arithmetic / 1 geometric sigma), FP64:
 * out[k][3 s + {0,1,2}] for k < slvmax (tagpt order) and solute site s. */
/* Intermediate-state extension (extensions/Intermediate/engproc.F90, solution mode):
 * refs_density[ermax] marks the zero-density bins (<= 1e-30); totals = {soln_total,
 * soln_intm, norm_intm}. */
int orc_intermediate_enable(orc_ctx* c, const double* refs_density);
int orc_intermediate_get(const orc_ctx* c, double* edintm, double* uvintm, double* totals);
int orc_adjoint(const orc_ctx* c, int tagslt, const double* solute_sitepos, int cmbrule, double* out);
int orc_recip_parts(const orc_ctx* c, int tagslt, const double* solute_sitepos, double* out,
                    double* self_out);
/* Direct Ewald reciprocal-space energy between the solute (positions xs, charges qs)
 * and every other molecule, summed over |m_i| <= mmax.  For PME validation. */
int orc_direct_ewald(const orc_ctx* c, int tagslt, const double* solute_sitepos, int mmax,
                     double* out /* (slvmax) */, double* self_out);

#ifdef __cplusplus
}
#endif
#endif
