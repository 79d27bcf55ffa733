// engine.cuh -- the context behind ermod_ctx (host side state + device buffers).
#pragma once

#include <cuda.h>  // CUtensorMap (types only; the encoder is fetched at run time)
#include <cufft.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/ermod_gpu.h"
#include "ermod_internal.cuh"

namespace ermod {

enum Phase { PH_FRAME = 0, PH_PREP, PH_SPECTRUM, PH_FFT, PH_GATHER, PH_MOL, PH_ACCUM, PH_ECORR, PH_ADJOINT, PH_COPY, PH_COUNT };
extern const char* const kPhaseNames[PH_COUNT];

struct Engine {
  ermod_params P{};
  int device = 0;
  int num_sm = 152;  // the device's SM count (launch shapes of the small kernels)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool mixed = true;
  int P_order = 4;

  // timing (CUDA events around each phase on the context's stream)
  bool timing = false;
  double phase_ms[PH_COUNT] = {};
  long long launches = 0;
  std::vector<cudaEvent_t> ev_pool;
  struct Pending { cudaEvent_t a, b; int phase; };
  std::vector<Pending> pending;
  // per stream: caller's, aux, prep, flush, the batch streams
  static_assert(4 + kBatchStreams <= 8, "phase slots per stream");
  int cur_phase[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
  cudaEvent_t cur_ev[8] = {};

  // ---- topology ----------------------------------------------------------------
  int nummol = 0, numatm = 0, ljtype_max = 0, slvmax = 0, nsite_phys = 0, max_mol_sites = 0;
  std::vector<int> mbi0;  // 0-based first atom of each molecule, nummol+1 entries
  std::vector<int> sluvid, uvspec, tagpt, numsite, ljtype0;
  std::vector<double> charge, mol_charge;
  double total_charge_phys = 0.0;
  bool topo_ready = false;
  double* d_charge = nullptr;
  int* d_ljtype = nullptr;       // 0-based
  double* d_ljene = nullptr;     // [T*T] column-major
  double* d_ljlensq = nullptr;
  float* d_ljene_f = nullptr;    // FP32 copies for the mixed pair terms
  float* d_ljlensq_f = nullptr;
  int* d_mol_atom0 = nullptr;    // [slvmax] first atom (0-based) of physical molecule k
  int* d_mol_nsite = nullptr;    // [slvmax]
  int* d_mol_species = nullptr;  // [slvmax] uvspec
  double* d_mol_qmol = nullptr;  // [slvmax]
  int* d_mbi0 = nullptr;         // [nummol+1] 0-based first atom of each molecule
  double* d_qmol_all = nullptr;  // [nummol] molecular charges
  int* d_mol_to_k = nullptr;     // [nummol] tagpt position (0-based) or -1

  // ---- energy coordinate ---------------------------------------------------------
  int numslv = 0, ermax = 0, esmax = 0;
  std::vector<int> uvmax, uvsoft, uvoff;
  std::vector<double> uvcrd, escrd;
  bool bins_ready = false;
  long long* d_uvkey = nullptr;  // ordered keys of uvcrd
  int* d_uvkey_f = nullptr;      // ordered 32-bit keys of uvcrd rounded down to floats (mixed binning)
  long long* d_eskey = nullptr;  // ordered keys of escrd
  int* d_spec = nullptr;         // [numslv][3] {uvoff, uvmax, uvsoft}

  // ---- accumulators ----------------------------------------------------------------
  double* d_edens = nullptr;
  double* d_ecorr = nullptr;
  long long* d_ecorr_n = nullptr;
  double* d_eself = nullptr;
  double* d_slnuv = nullptr;
  double* d_minuv = nullptr;  // [numslv+1]
  double* d_maxuv = nullptr;
  double* d_scal = nullptr;   // {engnorm, engsmpl, avslf, voffset, voffset_initialized, usreal, usreal_valid}
  bool warn_bin_firsttime = true;

  // ---- frame -----------------------------------------------------------------------
  FrameGeom geom{};
  double cell[9] = {}, prevcl[9] = {};
  bool green_valid = false, frame_ready = false;
  double stat_weight_system = 1.0;
  double* d_sitepos = nullptr;   // (3, numatm)
  double* d_engfac = nullptr;    // [K3][K2][H]
  float* d_engfac_f = nullptr;
  double* d_splfc = nullptr;     // [K1 + K2 + K3]
  float2* d_twiddle = nullptr;   // [K1 + K2 + K3] exp(-2 pi i m / K)
  double2* d_twiddle64 = nullptr;  // the same in FP64 (solute structure factors)
  double* d_wrapped = nullptr;   // (3, numatm) normalised coordinates
  // spatial sort of physical molecules
  unsigned int* d_sort_key = nullptr;
  unsigned int* d_sort_key_alt = nullptr;
  int* d_sort_val = nullptr;
  int* d_sort_val_alt = nullptr;
  void* d_cub_tmp = nullptr;
  size_t cub_tmp_bytes = 0;
  // slot-ordered solvent layout
  int* d_slot_mol = nullptr;      // [slvmax] tagpt index k held by slot m
  int* d_slot_site = nullptr;     // [slvmax+1] first site of slot m
  int* d_slot_species = nullptr;  // [slvmax]
  double* d_slot_qmol = nullptr;  // [slvmax]
  int4* d_site_pos = nullptr;     // [nsite_phys]
  float4* d_site_rec = nullptr;
  int* d_site_grid = nullptr;
  double* d_site_x = nullptr;     // [nsite_phys][3] FP64 wrapped coordinates (both paths)
  double* d_site_w = nullptr;     // FP64 path [nsite_phys][3][P]
  double* d_site_q = nullptr;     // [nsite_phys] FP64 charges (both paths)
  float* d_frame_scal = nullptr;  // [0] max molecule radius about its first site (A)
  // sites grouped by 8^3 bricks of the PME grid (the mixed gather's unit of work)
  int nbrick[3] = {1, 1, 1}, nbricks = 1;
  unsigned int* d_brick_key = nullptr;
  unsigned int* d_brick_key_alt = nullptr;
  int* d_brick_val = nullptr;
  int* d_brick_site = nullptr;   // [nsite_phys] site indices (slot order) sorted by brick
  int* d_brick_count = nullptr;  // [nbricks+1]
  int* d_brick_start = nullptr;  // [nbricks+1]

  // ---- batch buffers ---------------------------------------------------------------
  int Bmax = 1, G = 1, ntile = 1, tile = 256;
  int* d_tagslt = nullptr;        // [cap_place]
  double* d_solxyz = nullptr;     // [cap_place][S][3]
  double* d_sws = nullptr;        // [cap_place]
  int cap_place = 0;
  BatchArgs buf{};                // device buffers sized for Bmax (pointers only)
  // histogram ring for ecorr (corrcal) / per-batch histograms
  // histogram ring of the ecorr flush: two halves of ring_half entries; batches fill the
  // half at ring_off while the flush stream flushes the other one
  int ring_cap = 0, ring_fill = 0, ring_half = 0, ring_off = 0;
  bool flush_pend[2] = {false, false};  // a flush of that half may still be running
  int* d_ring_hist = nullptr;     // [ring_cap][ermax]
  double* d_ring_w = nullptr;     // [ring_cap]
  int* d_ring_nz = nullptr;       // ecorr flush scratch, [2][ring_cap][ermax]: the FP64 flush's occupied-bin
                                  // lists (bins, counts); the mixed flush's active-bin flags and list
  int* d_ring_nnz = nullptr;      // [ring_cap] occupied bins per entry
  int* d_ring_valid = nullptr;    // [ring_cap] entry accumulated (no error in its batch)
  double* d_u0 = nullptr;         // [2][Bmax] solute self energies (two batch slots)
  float* d_site_e = nullptr;      // [2][nsite_phys][Bmax] reciprocal site terms (mixed path)
  int* d_self_bin = nullptr;      // [2][Bmax]

  // ---- status ----------------------------------------------------------------------
  DevStatus* d_status = nullptr;
  DevStatus* h_status = nullptr;  // pinned
  int err_placement = -1, err_molecule = -1;
  double err_energy = 0.0;
  int call_b0 = 0;

  // ---- mixed path potential grids: padded periodic layout + TMA descriptor ----------
  int phi_dims[3] = {0, 0, 0};   // XP (multiple of 4), YP, ZP
  int gbox[3] = {0, 0, 0};       // gather box: x (multiple of 4), y, z
  CUtensorMap phi_tmap[kBatchSlots];  // per slot (the type carries its alignment)

  // adjoint mode (mixed path): bin-resolved derivatives of the solvent molecules'
  // energies with respect to the per-site charge, LJ epsilon and LJ sigma of a solute
  bool adj_on = false;
  int adj_mol = 0;      // 1-based molecule whose placements are differentiated
  int adj_ns = 0;       // its sites: 3 adj_ns parameters
  int adj_cmbrule = 0;  // sigma combination: 0 arithmetic, 1 geometric
  double* d_adj_grad = nullptr;  // [3 adj_ns][ermax] FP64 accumulators
  double* d_adj_w = nullptr;     // [ermax] weight of the molecules summed per bin
  float2* d_adj_par = nullptr;   // [adj_ns] {eps_s, sigma_s} of the solute sites
  float* d_adj_du = nullptr;     // [slvmax][3 adj_ns] per-molecule derivatives (one placement)
  int* d_adj_key = nullptr;      // [4][slvmax] bin keys and molecule slots, sorted copies
  int* d_adj_seg = nullptr;      // [2][ermax] segment begin / end in the sorted order
  void* d_adj_cub = nullptr;
  size_t adj_cub_bytes = 0;
  int* d_mol_bin = nullptr;      // [kBatchSlots][Bmax][slvmax] per-molecule bins (slot order)
  // unit-charge single-site "placements" whose potentials give d u / d q_s
  int* d_ps_nsite = nullptr;     // [Bmax]
  float* d_ps_qf = nullptr;      // [Bmax][256]
  float2* d_ps_bvec = nullptr;   // [Bmax][256][3][Kmax]
  double* d_ps_self = nullptr;   // [Bmax][K2]
  // host aggregate (hostspec) and reference structure (refspec + solute), both cleared by
  // ermod_set_topology
  double* d_agg_mass = nullptr;  // [numatm] site masses of the host aggregate (0 elsewhere)
  double* d_site_mass = nullptr; // [numatm] site masses of every molecule
  int ref_nh = 0, ref_ns = 0;    // reference host atoms and solute sites (ref_ns 0: none set)
  int* d_ref_atoms = nullptr;    // [ref_nh] 0-based atoms of the refspec molecules, in order
  double* d_ref_host = nullptr;  // [ref_nh][4] reference coordinates, weight
  double* d_ref_slt = nullptr;   // [ref_ns][4] reference solute coordinates, weight
  double* d_ref_fit = nullptr;   // generator: [256][3] starting structure, [256][3] fitted reference
                                 // solute (insorigin 3), or [3] the aggregate centre (insorigin 2)
  // solution-mode configuration check (check_mol_configuration): insposition 2-5 or 0
  // (no position test), insstructure 1 or 0
  int cfg_pos = 0, cfg_str = 0;
  double cfg_lw = 0.0, cfg_up = 0.0, cfg_lwstr = 0.0, cfg_upstr = 0.0;
  int* d_skip = nullptr;         // [cap_skip] 1: the placement is skipped
  int cap_skip = 0;
  unsigned char* d_int_mask = nullptr;  // intermediate state: [ermax] zero-density bins
  double* d_edintm = nullptr;            // [ermax] edintm, [numslv] uvintm, [3] totals
  double* d_ins = nullptr;       // [4][256] solute reference coordinates and masses (placement generator)
  // flexible solute (ermod_set_solute_library): SltConf's structures in file order, the
  // structure weights and the accepted structures (lib_nconf 0: no library)
  int lib_nconf = 0, lib_ns = 0, lib_nwt = 0, lib_na = 0;
  double* d_lib = nullptr;       // [lib_nconf][lib_ns][3]
  double* d_lib_wt = nullptr;    // [lib_nwt]
  int* d_lib_acc = nullptr;      // [lib_nconf] accepted structures in file order, their count at [lib_nconf]
  bool tmap_ready = false;

  // ---- cuFFT -------------------------------------------------------------------------
  cufftHandle plan_d2z = 0, plan_z2d = 0;
  bool plans_ready = false;

  // helpers
  int H() const { return geom.K[0] / 2 + 1; }
  size_t grid_real() const { return (size_t)geom.K[0] * geom.K[1] * geom.K[2]; }
  size_t grid_cplx() const { return (size_t)H() * geom.K[1] * geom.K[2]; }
  // FP32 engfac rows padded to a multiple of 4 points (16-byte loads in pme_a)
  int Hp4() const { return ((H() + 3) / 4) * 4; }
  int Kmax() const { return std::max(geom.K[0], std::max(geom.K[1], geom.K[2])); }

  // second stream: the ordered accumulation of batch i overlaps batch i+1's kernels;
  // third stream: the solute preparation of batch i+1 overlaps batch i's kernels
  cudaStream_t aux = nullptr;
  cudaStream_t prep = nullptr;
  // stream of the ecorr flushes (high priority, like aux): a flush only has to end before
  // its ring half is filled again, so the batch slots are freed without waiting for it
  cudaStream_t flush = nullptr;
  cudaEvent_t ev_prep[kBatchSlots] = {};  // preparation of the slot finished
  // mixed path: batches alternate between two streams (their PME grids and site terms
  // in kBatchSlots sets taken in turn), so one batch's kernels fill the other's partial
  // waves
  cudaStream_t bs[kBatchStreams] = {};
  cudaEvent_t ev_join[3 + kBatchStreams] = {};
  cudaEvent_t ev_done[kBatchSlots] = {};  // batch kernels finished (slot)
  cudaEvent_t ev_acc[kBatchSlots] = {};   // accumulation of the slot finished
  cudaEvent_t ev_flush[2] = {nullptr, nullptr};  // ecorr flush of ring half 0 / 1 finished

  void phase_begin(int ph) { phase_begin_on(ph, stream); }
  void phase_end() { phase_end_on(stream); }
  void phase_begin_on(int ph, cudaStream_t s);
  void phase_end_on(cudaStream_t s);
  int stream_index(cudaStream_t s) const {
    if (!s) return 0;
    if (s == aux) return 1;
    if (s == prep) return 2;
    if (s == flush) return 3;
    for (int k = 0; k < kBatchStreams; ++k)
      if (s == bs[k]) return 4 + k;
    return 0;
  }
  void count_launch(int n = 1) { launches += n; }
};

// sizes shared between the launchers and the host code
int spectrum_partials(const Engine& e);
int influence64_blocks();
int accumulate_max_batch();
size_t frame_cub_bytes(int n);
size_t brick_cub_bytes(int nsite, int nbricks);
cudaError_t launch_frame_bricks(Engine& e);
double host_spline_value(int order, double x);

// host utilities (engine.cu)
void set_error_string(const std::string& s);
int fail_cuda(cudaError_t e, const char* where);

}  // namespace ermod

#define ERMOD_CUDA(call)                                                              \
  do {                                                                                \
    cudaError_t err__ = (call);                                                       \
    if (err__ != cudaSuccess) return ::ermod::fail_cuda(err__, #call);                \
  } while (0)
