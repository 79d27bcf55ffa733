// engine.cu -- the C ABI (include/ermod_gpu.h): context life cycle, uploads, the
// per-frame preparation and the batched placement loop that replaces engconst's
// `do cntdst` (engproc.F90:388-392).
//
// Per batch of B placements:
//   [mixed] place_prep (prep stream) -> pme_a -> pme_b -> gather -> finish (one of two
//           batch streams) -> reduce + accumulate (aux stream)
//   [fp64]  place_prep -> spread64 -> D2Z -> influence64 -> Z2D -> mol_energy -> accumulate
// and, when ecorr is on, a flush of the histogram ring every `ring_half` placements on
// the flush stream while the next batches fill the ring's other half.
// Status is reported once per call (host API) or per ermod_sync (device API).
#include <cufft.h>

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.cuh"

namespace ermod {

const char* const kPhaseNames[PH_COUNT] = {"frame", "place_prep", "spectrum", "fft_c2r", "gather",
                                           "mol_energy", "accumulate", "ecorr", "adjoint", "copy"};

namespace {
thread_local std::string g_err;

template <typename T>
cudaError_t dalloc(T** p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return cudaMalloc((void**)p, sizeof(T) * n);
}
template <typename T>
void dfree(T*& p) {
  if (p) cudaFree((void*)p);
  p = nullptr;
}
}  // namespace

void set_error_string(const std::string& s) { g_err = s; }

int fail_cuda(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? ERMOD_E_NOMEM : ERMOD_E_CUDA;
}

static int fail_fft(cufftResult r, const char* where) {
  g_err = std::string(where) + ": cuFFT error " + std::to_string((int)r);
  return ERMOD_E_CUFFT;
}

static int fail_param(const char* what) {
  g_err = what;
  return ERMOD_E_PARAM;
}

void Engine::phase_begin_on(int ph, cudaStream_t s) {
  if (!timing) return;
  cudaEvent_t ev;
  if (!ev_pool.empty()) {
    ev = ev_pool.back();
    ev_pool.pop_back();
  } else {
    cudaEventCreate(&ev);
  }
  cudaEventRecord(ev, s);
  cur_phase[stream_index(s)] = ph;
  cur_ev[stream_index(s)] = ev;
}

void Engine::phase_end_on(cudaStream_t s) {
  const int si = stream_index(s);
  const int ph = cur_phase[si];
  if (!timing || ph < 0) return;
  cudaEvent_t ev;
  if (!ev_pool.empty()) {
    ev = ev_pool.back();
    ev_pool.pop_back();
  } else {
    cudaEventCreate(&ev);
  }
  cudaEventRecord(ev, s);
  pending.push_back(Pending{cur_ev[si], ev, ph});
  cur_phase[si] = -1;
  if (pending.size() > 8192) {  // harvest to bound the pool
    cudaEventSynchronize(ev);
    for (auto& p : pending) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, p.a, p.b);
      phase_ms[p.phase] += ms;
      ev_pool.push_back(p.a);
      ev_pool.push_back(p.b);
    }
    pending.clear();
  }
}

static void harvest(Engine& e) {
  if (e.pending.empty()) return;
  for (auto& p : e.pending) cudaEventSynchronize(p.b);
  for (auto& p : e.pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    e.phase_ms[p.phase] += ms;
    e.ev_pool.push_back(p.a);
    e.ev_pool.push_back(p.b);
  }
  e.pending.clear();
}

}  // namespace ermod

using namespace ermod;

struct ermod_ctx {
  Engine e;
};

// ---------------------------------------------------------------------------------
static int free_batch(Engine& e) {
  BatchArgs& b = e.buf;
  dfree(b.u_nsite);
  dfree(b.u_x);
  dfree(b.u_pos);
  dfree(b.u_q);
  dfree(b.u_qf);
  dfree(b.u_grid);
  dfree(b.u_w);
  dfree(b.u_bvec);
  dfree(b.u_qmol);
  dfree(b.u_usreal);
  dfree(b.u_radius);
  dfree(b.spec);
  dfree(b.phi);
  dfree(b.spec64);
  dfree(b.phi64);
  dfree(b.self_part);
  dfree(b.part);
  dfree(b.engnmfc);
  dfree(e.d_ring_hist);
  dfree(e.d_ring_w);
  dfree(e.d_ring_nz);
  dfree(e.d_ring_nnz);
  dfree(e.d_ring_valid);
  dfree(e.d_u0);
  dfree(e.d_site_e);
  dfree(e.d_self_bin);
  e.buf = BatchArgs{};
  return ERMOD_OK;
}

static int free_frame(Engine& e) {
  dfree(e.d_sitepos);
  dfree(e.d_wrapped);
  dfree(e.d_sort_key);
  dfree(e.d_sort_key_alt);
  dfree(e.d_sort_val);
  dfree(e.d_sort_val_alt);
  dfree(e.d_cub_tmp);
  dfree(e.d_slot_mol);
  dfree(e.d_slot_site);
  dfree(e.d_slot_species);
  dfree(e.d_slot_qmol);
  dfree(e.d_site_pos);
  dfree(e.d_site_rec);
  dfree(e.d_site_grid);
  dfree(e.d_site_x);
  dfree(e.d_site_w);
  dfree(e.d_site_q);
  dfree(e.d_frame_scal);
  dfree(e.d_brick_key);
  dfree(e.d_brick_key_alt);
  dfree(e.d_brick_val);
  dfree(e.d_brick_site);
  dfree(e.d_brick_count);
  dfree(e.d_brick_start);
  return ERMOD_OK;
}

static int free_topology(Engine& e) {
  dfree(e.d_charge);
  dfree(e.d_ljtype);
  dfree(e.d_ljene);
  dfree(e.d_ljlensq);
  dfree(e.d_ljene_f);
  dfree(e.d_ljlensq_f);
  dfree(e.d_mol_atom0);
  dfree(e.d_mol_nsite);
  dfree(e.d_mol_species);
  dfree(e.d_mol_qmol);
  dfree(e.d_mbi0);
  dfree(e.d_qmol_all);
  dfree(e.d_mol_to_k);
  return ERMOD_OK;
}

static int free_bins(Engine& e) {
  dfree(e.d_uvkey);
  dfree(e.d_uvkey_f);
  dfree(e.d_eskey);
  dfree(e.d_spec);
  dfree(e.d_edens);
  dfree(e.d_ecorr);
  dfree(e.d_ecorr_n);
  dfree(e.d_eself);
  dfree(e.d_slnuv);
  dfree(e.d_minuv);
  dfree(e.d_maxuv);
  dfree(e.d_scal);
  return ERMOD_OK;
}

// TMA descriptor of the padded potential grids, a 5-D tensor [B/4][ZP][YP][XP][4] (four
// placements interleaved innermost); one box = the gather halo of a brick for 4
// placements, landing in shared memory as [z][y][x][4]
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int make_phi_tmap(Engine& e, float* phi, CUtensorMap* map) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
  if (err != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
    g_err = "cuTensorMapEncodeTiled is not available";
    return ERMOD_E_CUDA;
  }
  const cuuint64_t XP = e.phi_dims[0], YP = e.phi_dims[1], ZP = e.phi_dims[2];
  const cuuint64_t dims[5] = {4, XP, YP, ZP, (cuuint64_t)((e.Bmax + 3) / 4)};
  const cuuint64_t strides[4] = {16, XP * 16, XP * YP * 16, XP * YP * ZP * 16};
  const cuuint32_t box[5] = {4, (cuuint32_t)e.gbox[0], (cuuint32_t)e.gbox[1], (cuuint32_t)e.gbox[2], 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = ((EncodeTiledFn)fn)(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, phi, dims, strides, box, estr,
                                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    g_err = "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")";
    return ERMOD_E_CUDA;
  }
  e.tmap_ready = true;
  return ERMOD_OK;
}

// batch buffers: need topology (slvmax), bins (ermax, numslv) and the PME grid
static int ensure_batch(Engine& e) {
  if (e.buf.u_nsite) return ERMOD_OK;
  const int S = kMaxSoluteSites;
  const int B = e.Bmax;
  BatchArgs& b = e.buf;
  const size_t nr = e.grid_real(), nc = e.grid_cplx();
  e.ntile = (e.slvmax + e.tile - 1) / e.tile;
  // solute data: kBatchSlots batch slots (the preparation of batch i+1 runs during batch i)
  const size_t NS = kBatchSlots;
  ERMOD_CUDA(dalloc(&b.u_nsite, NS * B));
  ERMOD_CUDA(dalloc(&b.u_x, NS * B * S * 3));
  ERMOD_CUDA(dalloc(&b.u_pos, NS * B * S));
  ERMOD_CUDA(dalloc(&b.u_q, NS * B * S));
  ERMOD_CUDA(dalloc(&b.u_qf, NS * B * S));
  ERMOD_CUDA(dalloc(&b.u_grid, NS * B * S));
  ERMOD_CUDA(dalloc(&b.u_w, NS * B * S * 3 * kMaxSplineOrder));
  ERMOD_CUDA(dalloc(&b.u_qmol, NS * B));
  ERMOD_CUDA(dalloc(&b.u_usreal, NS * B));
  ERMOD_CUDA(dalloc(&b.u_radius, NS * B));
  ERMOD_CUDA(dalloc(&b.engnmfc, NS * B));
  ERMOD_CUDA(dalloc(&e.d_u0, NS * B));
  ERMOD_CUDA(dalloc(&e.d_self_bin, NS * B));
  if (e.mixed) {
    ERMOD_CUDA(dalloc(&b.u_bvec, NS * B * S * 3 * e.Kmax()));
    // PME intermediate, padded potential grids and site terms: one set per batch slot
    ERMOD_CUDA(dalloc(&e.d_site_e, NS * e.nsite_phys * B));
    ERMOD_CUDA(dalloc(&b.spec, NS * nc * B));
    const int h = e.P_order - 1;
    e.phi_dims[0] = ((e.geom.K[0] + h + 3) / 4) * 4;
    e.phi_dims[1] = e.geom.K[1] + h;
    e.phi_dims[2] = e.geom.K[2] + h;
    // gather halo box: the brick plus the stencil reach below it, no wider (every element
    // is a 16-byte float4, so any x extent is a legal TMA box)
    e.gbox[0] = kBrickX + h;
    e.gbox[1] = kBrickY + h;
    e.gbox[2] = kBrickZ + h;
    const size_t np = (size_t)e.phi_dims[0] * e.phi_dims[1] * e.phi_dims[2];
    ERMOD_CUDA(dalloc(&b.phi, NS * np * B));
    ERMOD_CUDA(cudaMemset(b.phi, 0, sizeof(float) * NS * np * B));
    for (int s = 0; s < kBatchSlots; ++s) {
      const int st = make_phi_tmap(e, b.phi + (size_t)s * np * B, &e.phi_tmap[s]);
      if (st) return st;
    }
    ERMOD_CUDA(dalloc(&b.self_part, NS * B * spectrum_partials(e)));
  } else {
    ERMOD_CUDA(dalloc(&b.spec64, nc * B));
    ERMOD_CUDA(dalloc(&b.phi64, nr * B));
    ERMOD_CUDA(dalloc(&b.self_part, NS * B * influence64_blocks()));
  }
  ERMOD_CUDA(dalloc(&b.part, NS * B * e.ntile * e.numslv * 3));
  e.ring_half = e.P.corrcal ? std::max(2 * B, (512 / B) * B) : B;
  e.ring_cap = 2 * e.ring_half;
  e.ring_fill = 0;
  e.ring_off = 0;
  e.flush_pend[0] = e.flush_pend[1] = false;
  ERMOD_CUDA(dalloc(&e.d_ring_hist, (size_t)e.ring_cap * e.ermax));
  ERMOD_CUDA(dalloc(&e.d_ring_w, e.ring_cap));
  ERMOD_CUDA(dalloc(&e.d_ring_nnz, e.ring_cap));
  ERMOD_CUDA(dalloc(&e.d_ring_valid, e.ring_cap));
  if (e.P.corrcal) ERMOD_CUDA(dalloc(&e.d_ring_nz, (size_t)2 * e.ring_cap * e.ermax));
  // FFT plans
  if (!e.plans_ready) {
    int n[3] = {e.geom.K[2], e.geom.K[1], e.geom.K[0]};
    cufftResult r;
    if (!e.mixed) {
      r = cufftPlanMany(&e.plan_d2z, 3, n, nullptr, 1, (int)nr, nullptr, 1, (int)nc, CUFFT_D2Z, B);
      if (r != CUFFT_SUCCESS) return fail_fft(r, "cufftPlanMany(D2Z)");
      r = cufftPlanMany(&e.plan_z2d, 3, n, nullptr, 1, (int)nc, nullptr, 1, (int)nr, CUFFT_Z2D, B);
      if (r != CUFFT_SUCCESS) return fail_fft(r, "cufftPlanMany(Z2D)");
      cufftSetStream(e.plan_d2z, e.stream);
      cufftSetStream(e.plan_z2d, e.stream);
    }
    e.plans_ready = true;
  }
  return ERMOD_OK;
}

// ---------------------------------------------------------------------------------
extern "C" {

const char* ermod_last_error_string(void) { return g_err.c_str(); }

const char* ermod_status_string(int s) {
  switch (s) {
    case ERMOD_OK: return "ok";
    case ERMOD_E_ENG_MIN: return "eng_min: the minimum of the energy coordinate is too large";
    case ERMOD_E_ENG_SFT: return "eng_sft: energy beyond the soft region in the solution system";
    case ERMOD_E_ENG_BUG: return "eng_bug";
    case ERMOD_E_ENG_CNS: return "eng_cns: inconsistency in the species assignment";
    case ERMOD_E_RCP_CNS: return "rcp_cns: inconsistency in the reciprocal-space set-up";
    case ERMOD_E_RCP_FST: return "rcp_fst: the solute must not be a solvent";
    case ERMOD_E_INS_GEO: return "ins_geo: the system geometry is incorrectly set";
    case ERMOD_E_SET_PRS: return "set_prs: the system parameters are incorrectly set";
    case ERMOD_E_ENG_SLB: return "eng_slb: the slab configuration needs a periodic system";
    case ERMOD_W_MBIN: return "mbin: the maximum binning energy is too low for this species";
    case ERMOD_E_INS_SIZ: return "ins_siz: the solute structures differ in size";
    case ERMOD_E_PARAM: return "invalid argument";
    case ERMOD_E_NONCUBOID: return "a non-cuboidal cell is not supported";
    case ERMOD_E_UNSUPPORTED: return "unsupported mode";
    case ERMOD_E_CUDA: return "CUDA error";
    case ERMOD_E_CUFFT: return "cuFFT error";
    case ERMOD_E_NOMEM: return "device allocation failed";
    case ERMOD_E_DEVICE: return "device-side check failed";
    default: return "unknown status";
  }
}

void ermod_default_params(ermod_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->abi_version = ERMOD_ABI_VERSION;
  p->slttype = 1;
  p->estype = 2;
  p->cltype = 2;
  p->ljswitch = 0;
  p->splodr = 4;
  p->ms1max = p->ms2max = p->ms3max = 64;
  p->wgtslf = 0;
  p->corrcal = 0;
  p->selfcal = 0;
  p->force_calculation = 0;
  p->precision = ERMOD_PRECISION_MIXED;
  p->batch = 0;
  p->count_mirror = 0;
  p->elecut = 12.0;
  p->upljcut = 12.0;
  p->lwljcut = 10.0;
  p->screen = 0.0;
  p->temp = 300.0 * 8.314510e-3 / 4.184;
  p->block_threshold = 4.0;
  p->boxshp = 1;
  p->finish_group = 0;
}

int ermod_create(const ermod_params* p_in, int device, ermod_ctx** out) {
  if (!p_in || !out) return fail_param("null argument");
  *out = nullptr;
  // version 1 of the struct ends before boxshp: copy what it has, periodic system
  ermod_params pv{};
  if (p_in->abi_version == 1) {
    std::memcpy(&pv, p_in, offsetof(ermod_params, boxshp));
    pv.abi_version = ERMOD_ABI_VERSION;
    pv.boxshp = 1;
  } else if (p_in->abi_version == ERMOD_ABI_VERSION) {
    pv = *p_in;
  } else {
    return fail_param("abi_version mismatch");
  }
  const ermod_params* p = &pv;
  if (p->boxshp != 0 && p->boxshp != 1) return fail_param("boxshp must be 0 (non-periodic) or 1 (periodic)");
  if (p->boxshp == 0 && (p->estype == 2 || p->cltype != 0)) {  // setconf.F90:368-372
    g_err = "set_prs: a non-periodic system needs estype 1 (NVT) and cltype 0 (bare Coulomb)";
    return ERMOD_E_SET_PRS;
  }
  if (p->cltype != 0 && p->cltype != 2 && p->cltype != 3) {  // 1 (Ewald) stops in the reference (set_prs)
    g_err = "cltype 0 (bare Coulomb), 2 (PME) and 3 (PPPM) are implemented on the GPU";
    return ERMOD_E_UNSUPPORTED;
  }
  if (p->cltype == 3 && p->splodr % 2 == 1) return fail_param("interpolation order for PPPM must be even");
  if (p->slttype < 1 || p->slttype > 3) return fail_param("slttype must be 1, 2 or 3");
  if (p->finish_group != 0 && p->finish_group != 4 && p->finish_group != 8)
    return fail_param("finish_group must be 0 (automatic), 4 or 8");
  if (p->ljswitch < 0 || p->ljswitch > 3) return fail_param("ljswitch must be 0..3");
  if (p->splodr != 4 && p->splodr != 6 && p->splodr != 8) {
    g_err = "splodr must be 4, 6 or 8 on the GPU";
    return ERMOD_E_UNSUPPORTED;
  }
  const int K[3] = {p->ms1max, p->ms2max, p->ms3max};
  for (int i = 0; i < 3; ++i)
    if (K[i] < p->splodr || K[i] > 1000) return fail_param("PME grid sizes must lie in [splodr, 1000]");
  if (p->precision == ERMOD_PRECISION_MIXED && !pme_fits(K[0], K[1], K[2])) {
    g_err = "mixed precision: PME grid sizes must be products of 2, 3, 5 whose planes fit in shared memory";
    return ERMOD_E_UNSUPPORTED;
  }
  if (!(p->screen > 0) || !(p->temp > 0) || !(p->elecut > 0) || !(p->upljcut > 0) || !(p->lwljcut >= 0) ||
      p->lwljcut >= p->upljcut)
    return fail_param("screen, temp and cutoffs must be positive with lwljcut < upljcut");
  if (p->precision != ERMOD_PRECISION_FP64 && p->precision != ERMOD_PRECISION_MIXED)
    return fail_param("precision must be ERMOD_PRECISION_FP64 or ERMOD_PRECISION_MIXED");
  if (p->batch < 0 || p->batch > accumulate_max_batch() || (p->batch % 4) != 0)
    return fail_param("batch must be a multiple of 4 in [4, 512] (0 = automatic)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    g_err = "no CUDA device";
    return ERMOD_E_CUDA;
  }
  if (device < 0 || device >= ndev) return fail_param("device out of range");
  ERMOD_CUDA(cudaSetDevice(device));
  auto* c = new ermod_ctx();
  Engine& e = c->e;
  e.P = *p;
  e.device = device;
  e.mixed = p->precision == ERMOD_PRECISION_MIXED;
  e.P_order = p->splodr;
  e.geom.K[0] = K[0];
  e.geom.K[1] = K[1];
  e.geom.K[2] = K[2];
  e.Bmax = e.mixed ? (p->batch > 0 ? p->batch : 64) : 1;
  // four placements per molecule-energy block unless asked otherwise: measured 4% faster
  // than eight on the 33,000-water workload (fewer registers, more blocks in flight)
  e.G = e.mixed ? 4 : 1;
  if (e.mixed && e.P.finish_group == 8 && e.Bmax % 8 == 0) e.G = 8;
  int nsm = 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) == cudaSuccess && nsm > 0)
    e.num_sm = nsm;
  cudaError_t err = cudaStreamCreateWithFlags(&e.stream, cudaStreamNonBlocking);
  if (err != cudaSuccess) {
    delete c;
    return fail_cuda(err, "cudaStreamCreate");
  }
  e.own_stream = true;
  // the short kernels of the prep, aux and flush streams (solute preparation, ordered
  // accumulation, ecorr flush) take priority over the batch streams' pending blocks, so
  // the slots they free are not held up behind a whole PME launch
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if ((err = cudaStreamCreateWithPriority(&e.aux, cudaStreamNonBlocking, prio_hi)) != cudaSuccess ||
      (err = cudaStreamCreateWithPriority(&e.prep, cudaStreamNonBlocking, prio_hi)) != cudaSuccess ||
      (err = cudaStreamCreateWithPriority(&e.flush, cudaStreamNonBlocking, prio_hi)) != cudaSuccess) {
    ermod_destroy(c);
    return fail_cuda(err, "cudaStreamCreate");
  }
  for (int k = 0; k < kBatchStreams; ++k)
    if ((err = cudaStreamCreateWithFlags(&e.bs[k], cudaStreamNonBlocking)) != cudaSuccess) {
      ermod_destroy(c);
      return fail_cuda(err, "cudaStreamCreate");
    }
  for (int s = 0; s < kBatchSlots; ++s) {
    cudaEventCreateWithFlags(&e.ev_done[s], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&e.ev_acc[s], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&e.ev_prep[s], cudaEventDisableTiming);
  }
  cudaEventCreateWithFlags(&e.ev_flush[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&e.ev_flush[1], cudaEventDisableTiming);
  for (int s = 0; s < 3 + kBatchStreams; ++s) cudaEventCreateWithFlags(&e.ev_join[s], cudaEventDisableTiming);
  if ((err = dalloc(&e.d_status, 1)) != cudaSuccess || (err = cudaMallocHost(&e.h_status, sizeof(DevStatus))) != cudaSuccess) {
    ermod_destroy(c);
    return fail_cuda(err, "status allocation");
  }
  DevStatus s0{kNoError, kNoError, 0, 0};
  cudaMemcpy(e.d_status, &s0, sizeof(s0), cudaMemcpyHostToDevice);
  *e.h_status = s0;
  // splfc tables (init_spline_axis, recpcal.F90:87-109) and FFT twiddles
  std::vector<double> splfc;
  std::vector<float2> tw;
  std::vector<double2> tw64;
  for (int ax = 0; ax < 3; ++ax) {
    for (int rci = 0; rci < K[ax]; ++rci) {
      double re = 0.0, im = 0.0;
      for (int spi = 0; spi <= p->splodr - 2; ++spi) {
        const double chr = host_spline_value(p->splodr, (double)(spi + 1));
        const double rtp2 = 2.0 * kPi * (double)(spi * rci) / (double)K[ax];
        re += chr * std::cos(rtp2);
        im += chr * std::sin(rtp2);
      }
      splfc.push_back(re * re + im * im);
      const double ang = 2.0 * kPi * (double)rci / (double)K[ax];
      tw.push_back(make_float2((float)std::cos(ang), (float)(-std::sin(ang))));
      tw64.push_back(make_double2(std::cos(ang), -std::sin(ang)));
    }
  }
  if ((err = dalloc(&e.d_splfc, splfc.size())) != cudaSuccess || (err = dalloc(&e.d_twiddle, tw.size())) != cudaSuccess ||
      (err = dalloc(&e.d_twiddle64, tw64.size())) != cudaSuccess ||
      (err = dalloc(&e.d_engfac, e.grid_cplx())) != cudaSuccess ||
      (err = dalloc(&e.d_engfac_f, (size_t)e.Hp4() * e.geom.K[1] * e.geom.K[2])) != cudaSuccess ||
      (err = cudaMemset(e.d_engfac_f, 0, sizeof(float) * e.Hp4() * e.geom.K[1] * e.geom.K[2])) != cudaSuccess) {
    ermod_destroy(c);
    return fail_cuda(err, "PME tables");
  }
  cudaMemcpy(e.d_splfc, splfc.data(), sizeof(double) * splfc.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(e.d_twiddle, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(e.d_twiddle64, tw64.data(), sizeof(double2) * tw64.size(), cudaMemcpyHostToDevice);
  *out = c;
  return ERMOD_OK;
}

static void free_adjoint(Engine& e);
static void free_intermediate(Engine& e);
static void free_config_check(Engine& e);
static void free_library(Engine& e);

int ermod_destroy(ermod_ctx* c) {
  if (!c) return ERMOD_OK;
  Engine& e = c->e;
  cudaSetDevice(e.device);
  if (e.stream) cudaStreamSynchronize(e.stream);
  free_adjoint(e);
  free_intermediate(e);
  free_config_check(e);
  free_library(e);
  dfree(e.d_ins);
  free_batch(e);
  free_frame(e);
  free_topology(e);
  free_bins(e);
  dfree(e.d_engfac);
  dfree(e.d_engfac_f);
  dfree(e.d_splfc);
  dfree(e.d_twiddle);
  dfree(e.d_twiddle64);
  dfree(e.d_status);
  if (e.h_status) cudaFreeHost(e.h_status);
  if (e.plan_d2z) cufftDestroy(e.plan_d2z);
  if (e.plan_z2d) cufftDestroy(e.plan_z2d);
  harvest(e);
  for (auto ev : e.ev_pool) cudaEventDestroy(ev);
  if (e.own_stream && e.stream) cudaStreamDestroy(e.stream);
  if (e.aux) cudaStreamSynchronize(e.aux);
  if (e.prep) cudaStreamSynchronize(e.prep);
  if (e.flush) cudaStreamSynchronize(e.flush);
  for (int s = 0; s < kBatchStreams; ++s)
    if (e.bs[s]) cudaStreamSynchronize(e.bs[s]);
  for (int s = 0; s < kBatchSlots; ++s) {
    if (e.ev_done[s]) cudaEventDestroy(e.ev_done[s]);
    if (e.ev_acc[s]) cudaEventDestroy(e.ev_acc[s]);
    if (e.ev_prep[s]) cudaEventDestroy(e.ev_prep[s]);
  }
  for (int s = 0; s < 2; ++s)
    if (e.ev_flush[s]) cudaEventDestroy(e.ev_flush[s]);
  if (e.aux) cudaStreamDestroy(e.aux);
  if (e.prep) cudaStreamDestroy(e.prep);
  if (e.flush) cudaStreamDestroy(e.flush);
  for (int s = 0; s < kBatchStreams; ++s)
    if (e.bs[s]) cudaStreamDestroy(e.bs[s]);
  for (int s = 0; s < 3 + kBatchStreams; ++s)
    if (e.ev_join[s]) cudaEventDestroy(e.ev_join[s]);
  delete c;
  return ERMOD_OK;
}

int ermod_set_stream(ermod_ctx* c, void* stream) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  if (e.stream) cudaStreamSynchronize(e.stream);
  if (e.own_stream && e.stream) cudaStreamDestroy(e.stream);
  e.stream = (cudaStream_t)stream;
  e.own_stream = false;
  if (e.plan_d2z) cufftSetStream(e.plan_d2z, e.stream);
  if (e.plan_z2d) cufftSetStream(e.plan_z2d, e.stream);
  return ERMOD_OK;
}

int ermod_set_topology(ermod_ctx* c, int nummol, int numatm, const int* mbi, const int* sluvid, const int* uvspec,
                       const double* charge, const int* ljtype, int ljtype_max, const double* ljene,
                       const double* ljlensq) {
  if (!c || !mbi || !sluvid || !uvspec || !charge || !ljtype || !ljene || !ljlensq) return fail_param("null argument");
  if (nummol <= 0 || numatm <= 0 || ljtype_max <= 0) return fail_param("sizes must be positive");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  cudaStreamSynchronize(e.stream);
  free_adjoint(e);  // sized by the topology: enable it again afterwards
  free_config_check(e);
  if (mbi[0] != 1 || mbi[nummol] - 1 != numatm) return fail_param("mol_begin_index must run from 1 to numatm+1");
  for (int i = 0; i < nummol; ++i) {
    if (mbi[i + 1] <= mbi[i]) return fail_param("every molecule needs at least one site");
    if (sluvid[i] < 0 || sluvid[i] > 3) return ERMOD_E_ENG_BUG;  // sanity_check_sluvid, engproc.F90:1023-1043
  }
  for (int a = 0; a < numatm; ++a)
    if (ljtype[a] < 1 || ljtype[a] > ljtype_max) return fail_param("ljtype out of range");
  // sanity_check_sluvid per slttype
  bool any_solute = false, any_solvent = false;
  for (int i = 0; i < nummol; ++i) {
    any_solute |= sluvid[i] != 0;
    any_solvent |= sluvid[i] == 0;
    if (e.P.slttype == 1 && sluvid[i] >= 2) {
      g_err = "eng_par: solution mode needs sluvid 0 or 1";
      return ERMOD_E_PARAM;
    }
    if (e.P.slttype != 1 && sluvid[i] == 1) {
      g_err = "eng_par: reference mode needs sluvid 0, 2 or 3";
      return ERMOD_E_PARAM;
    }
  }
  if (!any_solute || (e.P.slttype != 1 && !any_solvent)) {
    g_err = "eng_par: solute and solvent must both exist";
    return ERMOD_E_PARAM;
  }
  free_batch(e);
  free_frame(e);
  free_topology(e);
  e.frame_ready = false;
  e.topo_ready = false;
  e.nummol = nummol;
  e.numatm = numatm;
  e.ljtype_max = ljtype_max;
  e.mbi0.assign(nummol + 1, 0);
  for (int i = 0; i <= nummol; ++i) e.mbi0[i] = mbi[i] - 1;
  e.sluvid.assign(sluvid, sluvid + nummol);
  e.uvspec.assign(uvspec, uvspec + nummol);
  e.charge.assign(charge, charge + numatm);
  e.ljtype0.resize(numatm);
  for (int a = 0; a < numatm; ++a) e.ljtype0[a] = ljtype[a] - 1;
  e.numsite.resize(nummol);
  e.mol_charge.assign(nummol, 0.0);
  e.tagpt.clear();
  std::vector<int> mol_to_k(nummol, -1);
  e.total_charge_phys = 0.0;
  e.max_mol_sites = 0;
  for (int i = 0; i < nummol; ++i) {
    e.numsite[i] = e.mbi0[i + 1] - e.mbi0[i];
    double s = 0.0;  // mol_charge (setconf.F90:832-834)
    for (int a = e.mbi0[i]; a < e.mbi0[i + 1]; ++a) s += charge[a];
    e.mol_charge[i] = s;
    if (sluvid[i] == 0 || sluvid[i] == 1) {  // tagpt (engproc.F90:336-348)
      mol_to_k[i] = (int)e.tagpt.size();
      e.tagpt.push_back(i);
      e.max_mol_sites = std::max(e.max_mol_sites, e.numsite[i]);
    }
  }
  // volcorrect's charge sum in the reference's order (engproc.F90:880-881)
  for (int i = 0; i < nummol; ++i)
    if (sluvid[i] == 0 || sluvid[i] == 1) e.total_charge_phys += e.mol_charge[i];
  e.slvmax = (int)e.tagpt.size();
  if (e.slvmax == 0) return fail_param("no physical molecules");
  std::vector<int> atom0(e.slvmax), nsite(e.slvmax), species(e.slvmax);
  std::vector<double> qmol(e.slvmax);
  e.nsite_phys = 0;
  for (int k = 0; k < e.slvmax; ++k) {
    const int i = e.tagpt[k];
    atom0[k] = e.mbi0[i];
    nsite[k] = e.numsite[i];
    species[k] = uvspec[i];
    qmol[k] = e.mol_charge[i];
    e.nsite_phys += nsite[k];
  }
  std::vector<double> lje(ljene, ljene + (size_t)ljtype_max * ljtype_max);
  std::vector<double> ljl(ljlensq, ljlensq + (size_t)ljtype_max * ljtype_max);
  ERMOD_CUDA(dalloc(&e.d_charge, numatm));
  ERMOD_CUDA(dalloc(&e.d_ljtype, numatm));
  ERMOD_CUDA(dalloc(&e.d_ljene, lje.size()));
  ERMOD_CUDA(dalloc(&e.d_ljlensq, ljl.size()));
  ERMOD_CUDA(dalloc(&e.d_mol_atom0, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_mol_nsite, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_mol_species, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_mol_qmol, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_mbi0, nummol + 1));
  ERMOD_CUDA(dalloc(&e.d_qmol_all, nummol));
  ERMOD_CUDA(dalloc(&e.d_mol_to_k, nummol));
  ERMOD_CUDA(cudaMemcpy(e.d_charge, charge, sizeof(double) * numatm, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_ljtype, e.ljtype0.data(), sizeof(int) * numatm, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_ljene, lje.data(), sizeof(double) * lje.size(), cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_ljlensq, ljl.data(), sizeof(double) * ljl.size(), cudaMemcpyHostToDevice));
  {
    std::vector<float> fe(lje.begin(), lje.end()), fl(ljl.begin(), ljl.end());
    ERMOD_CUDA(dalloc(&e.d_ljene_f, fe.size()));
    ERMOD_CUDA(dalloc(&e.d_ljlensq_f, fl.size()));
    ERMOD_CUDA(cudaMemcpy(e.d_ljene_f, fe.data(), sizeof(float) * fe.size(), cudaMemcpyHostToDevice));
    ERMOD_CUDA(cudaMemcpy(e.d_ljlensq_f, fl.data(), sizeof(float) * fl.size(), cudaMemcpyHostToDevice));
  }
  ERMOD_CUDA(cudaMemcpy(e.d_mol_atom0, atom0.data(), sizeof(int) * e.slvmax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_mol_nsite, nsite.data(), sizeof(int) * e.slvmax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_mol_species, species.data(), sizeof(int) * e.slvmax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_mol_qmol, qmol.data(), sizeof(double) * e.slvmax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_mbi0, e.mbi0.data(), sizeof(int) * (nummol + 1), cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_qmol_all, e.mol_charge.data(), sizeof(double) * nummol, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_mol_to_k, mol_to_k.data(), sizeof(int) * nummol, cudaMemcpyHostToDevice));
  // frame buffers
  ERMOD_CUDA(dalloc(&e.d_sitepos, 3 * (size_t)numatm));
  ERMOD_CUDA(dalloc(&e.d_wrapped, 3 * (size_t)numatm));
  ERMOD_CUDA(dalloc(&e.d_sort_key, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_sort_key_alt, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_sort_val, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_sort_val_alt, e.slvmax + 1));
  ERMOD_CUDA(cudaMemset(e.d_sort_val_alt, 0, sizeof(int) * (e.slvmax + 1)));
  e.nbrick[0] = (e.geom.K[0] + kBrickX - 1) / kBrickX;
  e.nbrick[1] = (e.geom.K[1] + kBrickY - 1) / kBrickY;
  e.nbrick[2] = (e.geom.K[2] + kBrickZ - 1) / kBrickZ;
  e.nbricks = e.nbrick[0] * e.nbrick[1] * e.nbrick[2];
  e.cub_tmp_bytes = std::max(frame_cub_bytes(e.slvmax), brick_cub_bytes(e.nsite_phys, e.nbricks));
  ERMOD_CUDA(dalloc((char**)&e.d_cub_tmp, e.cub_tmp_bytes));
  ERMOD_CUDA(dalloc(&e.d_slot_mol, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_slot_site, e.slvmax + 1));
  ERMOD_CUDA(dalloc(&e.d_slot_species, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_slot_qmol, e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_site_pos, e.nsite_phys));
  ERMOD_CUDA(dalloc(&e.d_site_grid, e.nsite_phys));
  if (e.mixed) {
    ERMOD_CUDA(dalloc(&e.d_site_rec, e.nsite_phys));
    ERMOD_CUDA(dalloc(&e.d_brick_key, e.nsite_phys));
    ERMOD_CUDA(dalloc(&e.d_brick_key_alt, e.nsite_phys));
    ERMOD_CUDA(dalloc(&e.d_brick_val, e.nsite_phys));
    ERMOD_CUDA(dalloc(&e.d_brick_site, e.nsite_phys));
    ERMOD_CUDA(dalloc(&e.d_brick_count, e.nbricks + 1));
    ERMOD_CUDA(dalloc(&e.d_brick_start, e.nbricks + 1));
  } else {
    ERMOD_CUDA(dalloc(&e.d_site_w, (size_t)e.nsite_phys * 3 * e.P_order));
  }
  ERMOD_CUDA(dalloc(&e.d_site_x, 3 * (size_t)e.nsite_phys));
  ERMOD_CUDA(dalloc(&e.d_site_q, e.nsite_phys));
  ERMOD_CUDA(dalloc(&e.d_frame_scal, 4));
  e.green_valid = false;
  e.topo_ready = true;
  return ERMOD_OK;
}

int ermod_set_bins(ermod_ctx* c, int numslv, const int* uvmax, const int* uvsoft, const double* uvcrd, int esmax,
                   const double* escrd) {
  if (!c || !uvmax || !uvsoft || !uvcrd) return fail_param("null argument");
  if (numslv <= 0 || numslv > kMaxSpecies) return fail_param("numslv out of range");
  if (esmax < 0 || (esmax > 0 && !escrd)) return fail_param("escrd missing");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  cudaStreamSynchronize(e.stream);
  free_adjoint(e);  // sized by the bins: enable it again afterwards
  free_intermediate(e);
  int ermax = 0;
  for (int s = 0; s < numslv; ++s) {
    if (uvmax[s] <= 0 || uvsoft[s] < 0 || uvsoft[s] > uvmax[s]) return fail_param("uvmax/uvsoft inconsistent");
    ermax += uvmax[s];
  }
  // binsearch (engproc.F90:927-957) needs each species' edges in increasing order
  for (int sp = 0, off = 0; sp < numslv; off += uvmax[sp], ++sp)
    for (int i = off; i < off + uvmax[sp]; ++i)
      if (!(uvcrd[i] == uvcrd[i]) || (i > off && !(uvcrd[i] > uvcrd[i - 1])))
        return fail_param("uvcrd must increase within each species");
  free_batch(e);
  free_bins(e);
  e.bins_ready = false;
  e.numslv = numslv;
  e.ermax = ermax;
  e.esmax = esmax;
  e.uvmax.assign(uvmax, uvmax + numslv);
  e.uvsoft.assign(uvsoft, uvsoft + numslv);
  e.uvoff.assign(numslv, 0);
  std::vector<int> spec(3 * numslv);
  int off = 0;
  for (int s = 0; s < numslv; ++s) {
    e.uvoff[s] = off;
    spec[3 * s] = off;
    spec[3 * s + 1] = uvmax[s];
    spec[3 * s + 2] = uvsoft[s];
    off += uvmax[s];
  }
  e.uvcrd.assign(uvcrd, uvcrd + ermax);
  e.escrd.assign(escrd ? escrd : uvcrd, (escrd ? escrd : uvcrd) + esmax);
  std::vector<long long> uk(ermax), ek(std::max(esmax, 1));
  std::vector<int> ukf(ermax);
  for (int i = 0; i < ermax; ++i) {
    uk[i] = ordered_key(uvcrd[i]);
    float f = (float)uvcrd[i];  // round down to a float
    if ((double)f > uvcrd[i]) f = std::nextafter(f, -INFINITY);
    ukf[i] = ordered_key32(f);
  }
  for (int i = 0; i < esmax; ++i) ek[i] = ordered_key(escrd[i]);
  ERMOD_CUDA(dalloc(&e.d_uvkey, ermax));
  ERMOD_CUDA(dalloc(&e.d_eskey, ek.size()));
  ERMOD_CUDA(dalloc(&e.d_spec, spec.size()));
  ERMOD_CUDA(cudaMemcpy(e.d_uvkey, uk.data(), sizeof(long long) * ermax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(dalloc(&e.d_uvkey_f, ermax));
  ERMOD_CUDA(cudaMemcpy(e.d_uvkey_f, ukf.data(), sizeof(int) * ermax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_eskey, ek.data(), sizeof(long long) * ek.size(), cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_spec, spec.data(), sizeof(int) * spec.size(), cudaMemcpyHostToDevice));
  ERMOD_CUDA(dalloc(&e.d_edens, ermax));
  if (e.P.corrcal) {
    ERMOD_CUDA(dalloc(&e.d_ecorr, (size_t)ermax * ermax));
    if (e.P.count_mirror) ERMOD_CUDA(dalloc(&e.d_ecorr_n, (size_t)ermax * ermax));
  }
  ERMOD_CUDA(dalloc(&e.d_eself, std::max(esmax, 1)));
  ERMOD_CUDA(dalloc(&e.d_slnuv, numslv));
  ERMOD_CUDA(dalloc(&e.d_minuv, numslv + 1));
  ERMOD_CUDA(dalloc(&e.d_maxuv, numslv + 1));
  ERMOD_CUDA(dalloc(&e.d_scal, 8));
  // enginit's initial values (engproc.F90:255-260): minuv = infty, maxuv = -infty, voffset = -infty
  std::vector<double> mn(numslv + 1, 1.0e50), mx(numslv + 1, -1.0e50);
  ERMOD_CUDA(cudaMemcpy(e.d_minuv, mn.data(), sizeof(double) * (numslv + 1), cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_maxuv, mx.data(), sizeof(double) * (numslv + 1), cudaMemcpyHostToDevice));
  const double scal[8] = {0.0, 0.0, 0.0, -1.0e50, 0.0, 0.0, 0.0, 0.0};
  ERMOD_CUDA(cudaMemcpy(e.d_scal, scal, sizeof(scal), cudaMemcpyHostToDevice));
  if (e.P.corrcal) {
    ERMOD_CUDA(cudaMemset(e.d_ecorr, 0, sizeof(double) * (size_t)ermax * ermax));
    if (e.d_ecorr_n) ERMOD_CUDA(cudaMemset(e.d_ecorr_n, 0, sizeof(long long) * (size_t)ermax * ermax));
  }
  ERMOD_CUDA(cudaMemset(e.d_edens, 0, sizeof(double) * ermax));
  ERMOD_CUDA(cudaMemset(e.d_eself, 0, sizeof(double) * std::max(esmax, 1)));
  ERMOD_CUDA(cudaMemset(e.d_slnuv, 0, sizeof(double) * numslv));
  e.warn_bin_firsttime = true;
  e.bins_ready = true;
  return ERMOD_OK;
}

static int frame_common(Engine& e, const double* cell, double sws, double extent) {
  if (e.P.boxshp == 0) {
    // non-periodic: the cell is not used (NVT, bare Coulomb).  The fixed-point
    // coordinates and the spatial sort take a virtual cube, a power of two at least
    // 8 x the largest |coordinate|, so that pair differences of the frame's sites and of
    // solute sites within `reach` of the origin stay below half of it
    if (!std::isfinite(extent)) return fail_param("non-finite coordinates");
    std::memcpy(e.cell, cell, sizeof(double) * 9);
    e.stat_weight_system = sws;
    FrameGeom& g = e.geom;
    const double ext = std::max(extent, 16.0);
    double Lv = 128.0;
    while (Lv < 8.0 * ext) Lv *= 2.0;
    for (int i = 0; i < 9; ++i) g.invcl[i] = 0.0;
    for (int i = 0; i < 3; ++i) {
      g.L[i] = Lv;
      g.invL[i] = 1.0 / Lv;
      g.fx_scale[i] = Lv / 4294967296.0;
      g.invcl[4 * i] = 1.0 / Lv;
    }
    g.volume = Lv * Lv * Lv;
    g.periodic = 0;
    g.reach = 0.5 * Lv - ext;
    return ERMOD_OK;
  }
  // cuboid cells only (realcal.F90:859-866); lower off-diagonals too, since the QR
  // rotation of normalize_periodic is not applied
  if (std::fabs(cell[3]) > 1e-8 || std::fabs(cell[6]) > 1e-8 || std::fabs(cell[7]) > 1e-8 ||
      std::fabs(cell[1]) > 1e-8 || std::fabs(cell[2]) > 1e-8 || std::fabs(cell[5]) > 1e-8 || !(cell[0] > 0) ||
      !(cell[4] > 0) || !(cell[8] > 0)) {
    g_err = "A non-cuboidal cell is not supported";
    return ERMOD_E_NONCUBOID;
  }
  std::memcpy(e.cell, cell, sizeof(double) * 9);
  e.stat_weight_system = sws;
  FrameGeom& g = e.geom;
  // get_inverted_cell (engproc.F90:898-919)
  auto C = [&](int i, int j) { return cell[(i - 1) + 3 * (j - 1)]; };
  const double v = C(1, 1) * C(2, 2) * C(3, 3) + C(1, 2) * C(2, 3) * C(3, 1) + C(1, 3) * C(2, 1) * C(3, 2) -
                   C(1, 3) * C(2, 2) * C(3, 1) - C(1, 2) * C(2, 1) * C(3, 3) - C(1, 1) * C(2, 3) * C(3, 2);
  double ic[9];
  ic[0] = C(2, 2) * C(3, 3) - C(2, 3) * C(3, 2);
  ic[3] = C(1, 3) * C(3, 2) - C(1, 2) * C(3, 3);
  ic[6] = C(1, 2) * C(2, 3) - C(1, 3) * C(2, 2);
  ic[1] = C(2, 3) * C(3, 1) - C(2, 1) * C(3, 3);
  ic[4] = C(1, 1) * C(3, 3) - C(1, 3) * C(3, 1);
  ic[7] = C(1, 3) * C(2, 1) - C(1, 1) * C(2, 3);
  ic[2] = C(2, 1) * C(3, 2) - C(2, 2) * C(3, 1);
  ic[5] = C(1, 2) * C(3, 1) - C(1, 1) * C(3, 2);
  ic[8] = C(1, 1) * C(2, 2) - C(1, 2) * C(2, 1);
  for (int i = 0; i < 9; ++i) g.invcl[i] = ic[i] / v;
  g.volume = v;
  for (int i = 0; i < 3; ++i) {
    g.L[i] = std::fabs(cell[4 * i]);
    g.invL[i] = 1.0 / g.L[i];
    g.fx_scale[i] = g.L[i] / 4294967296.0;
  }
  g.periodic = 1;
  g.reach = 0.0;
  return ERMOD_OK;
}

static int frame_launch(Engine& e) {
  e.phase_begin(PH_FRAME);
  bool changed = !e.green_valid;
  for (int i = 0; i < 9; ++i) changed = changed || (e.prevcl[i] != e.cell[i]);
  if (changed && e.P.cltype != 0) ERMOD_CUDA(launch_greenfunc(e));
  std::memcpy(e.prevcl, e.cell, sizeof(e.cell));
  e.green_valid = true;
  ERMOD_CUDA(launch_frame_wrap(e));
  ERMOD_CUDA(launch_frame_sort(e));
  ERMOD_CUDA(launch_frame_sites(e));
  if (e.mixed) ERMOD_CUDA(launch_frame_bricks(e));
  e.phase_end();
  e.frame_ready = true;
  return ERMOD_OK;
}

int ermod_frame(ermod_ctx* c, const double* sitepos, const double* cell, double sws) {
  if (!c || !sitepos || !cell) return fail_param("null argument");
  Engine& e = c->e;
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  cudaSetDevice(e.device);
  double extent = 0.0;
  if (e.P.boxshp == 0) {
    bool finite = true;
    for (size_t i = 0; i < 3 * (size_t)e.numatm; ++i) {
      finite = finite && std::isfinite(sitepos[i]);
      extent = std::max(extent, std::fabs(sitepos[i]));
    }
    if (!finite) extent = std::nan("");
  }
  int st = frame_common(e, cell, sws, extent);
  if (st) return st;
  ERMOD_CUDA(cudaMemcpyAsync(e.d_sitepos, sitepos, sizeof(double) * 3 * e.numatm, cudaMemcpyHostToDevice, e.stream));
  st = frame_launch(e);
  if (st) return st;
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  return ERMOD_OK;
}

int ermod_frame_device(ermod_ctx* c, const double* sitepos_d, const double* cell, double sws) {
  if (!c || !sitepos_d || !cell) return fail_param("null argument");
  Engine& e = c->e;
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  cudaSetDevice(e.device);
  double extent = 0.0;
  if (e.P.boxshp == 0) ERMOD_CUDA(launch_max_abs(e, sitepos_d, 3 * (size_t)e.numatm, &extent));
  int st = frame_common(e, cell, sws, extent);
  if (st) return st;
  ERMOD_CUDA(cudaMemcpyAsync(e.d_sitepos, sitepos_d, sizeof(double) * 3 * e.numatm, cudaMemcpyDeviceToDevice,
                             e.stream));
  return frame_launch(e);
}

// the placement loop on device-resident inputs.  Batch i runs its kernels on batch stream
// i%2 with the buffers of slot i%kBatchSlots.  Its solute preparation runs on the prep stream
// during batch i-1; its ordered accumulation runs on the aux stream during batch i+1 and,
// every ring_half placements, the ecorr flush on the flush stream after it.
static int run_placements(Engine& e, int nplace, const int* d_tag, const double* d_sol, const double* d_sws,
                          double* d_uv, double* d_fl, int ns_solute) {
  int st = ensure_batch(e);
  if (st) return st;
  const int B = e.Bmax;
  const int S = kMaxSoluteSites;
  const int nbatch = (nplace + B - 1) / B;
  const size_t parts = e.mixed ? (size_t)spectrum_partials(e) : (size_t)influence64_blocks();
  // batches run on two alternating streams (mixed path) or on the caller's stream (FP64
  // path, whose cuFFT plans are bound to it); every stream starts after what is
  // already queued on the caller's stream
  const bool dual = e.mixed;
  // solution mode: the placements check_mol_configuration skips (engproc.F90:389-390)
  const bool check = e.P.slttype == 1 && (e.cfg_pos != 0 || e.cfg_str != 0) && nplace > 0;
  if (check) {
    if (nplace > e.cap_skip) {
      dfree(e.d_skip);
      e.cap_skip = nplace;
      ERMOD_CUDA(dalloc(&e.d_skip, (size_t)e.cap_skip));
    }
    ERMOD_CUDA(launch_config_check(e, nplace, d_tag));
  }
  ERMOD_CUDA(cudaEventRecord(e.ev_done[0], e.stream));
  ERMOD_CUDA(cudaStreamWaitEvent(e.aux, e.ev_done[0], 0));
  ERMOD_CUDA(cudaStreamWaitEvent(e.prep, e.ev_done[0], 0));
  if (dual) {
    for (int k = 0; k < kBatchStreams; ++k) ERMOD_CUDA(cudaStreamWaitEvent(e.bs[k], e.ev_done[0], 0));
  }
  auto batch_args = [&](int ib) {
    const int b0 = ib * B, slot = ib % kBatchSlots;
    BatchArgs a = e.buf;
    a.nb = std::min(B, nplace - b0);
    a.b0 = b0;
    a.G = e.G;
    a.tagslt = d_tag + b0;
    a.stat_weight_solute = d_sws ? d_sws + b0 : nullptr;
    a.uvengy_out = d_uv;
    a.flceng_out = d_fl;
    a.u_nsite = e.buf.u_nsite + (size_t)slot * B;
    a.u_x = e.buf.u_x + (size_t)slot * B * S * 3;
    a.u_pos = e.buf.u_pos + (size_t)slot * B * S;
    a.u_q = e.buf.u_q + (size_t)slot * B * S;
    a.u_qf = e.buf.u_qf + (size_t)slot * B * S;
    a.u_grid = e.buf.u_grid + (size_t)slot * B * S;
    a.u_w = e.buf.u_w + (size_t)slot * B * S * 3 * kMaxSplineOrder;
    if (e.buf.u_bvec) a.u_bvec = e.buf.u_bvec + (size_t)slot * B * S * 3 * e.Kmax();
    a.u_radius = e.buf.u_radius + (size_t)slot * B;
    a.u_qmol = e.buf.u_qmol + (size_t)slot * B;
    a.u_usreal = e.buf.u_usreal + (size_t)slot * B;
    a.engnmfc = e.buf.engnmfc + (size_t)slot * B;
    a.self_part = e.buf.self_part + (size_t)slot * B * parts;
    a.part = e.buf.part + (size_t)slot * B * e.ntile * e.numslv * 3;
    a.u0 = e.d_u0 + (size_t)slot * B;
    a.self_bin = e.d_self_bin + (size_t)slot * B;
    a.slot = slot;
    a.stream = dual ? e.bs[ib % kBatchStreams] : e.stream;  // streams and slots taken in turn
    a.phases = 1;
    a.mol_bin = e.adj_on ? e.d_mol_bin + (size_t)slot * B * e.slvmax : nullptr;
    a.skip = check ? e.d_skip + b0 : nullptr;
    if (e.mixed) {
      const size_t np = (size_t)e.phi_dims[0] * e.phi_dims[1] * e.phi_dims[2];
      a.spec = e.buf.spec + (size_t)slot * e.grid_cplx() * B;
      a.phi = e.buf.phi + (size_t)slot * np * B;
      a.site_e = e.d_site_e + (size_t)slot * e.nsite_phys * B;
    }
    return a;
  };
  auto issue_prep = [&](int ib) -> int {
    const int slot = ib % kBatchSlots;
    const BatchArgs a = batch_args(ib);
    if (ib >= kBatchSlots) ERMOD_CUDA(cudaStreamWaitEvent(e.prep, e.ev_acc[slot], 0));  // slot free again
    const double* sol = d_sol ? d_sol + (size_t)a.b0 * ns_solute * 3 : nullptr;
    e.phase_begin_on(PH_PREP, e.prep);
    ERMOD_CUDA(launch_place_prep(e, a, sol, e.P.slttype == 2 ? 2 : 1, e.prep));
    e.phase_end_on(e.prep);
    ERMOD_CUDA(cudaEventRecord(e.ev_prep[slot], e.prep));
    return ERMOD_OK;
  };
  if (nbatch > 0 && (st = issue_prep(0)) != ERMOD_OK) return st;
  for (int ibatch = 0; ibatch < nbatch; ++ibatch) {
    const int slot = ibatch % kBatchSlots;
    if (ibatch + 1 < nbatch && (st = issue_prep(ibatch + 1)) != ERMOD_OK) return st;
    BatchArgs a = batch_args(ibatch);
    const int nb = a.nb;
    a.hist = e.d_ring_hist + (size_t)(e.ring_off + e.ring_fill) * e.ermax;
    cudaStream_t bst = a.stream;
    if (ibatch >= kBatchSlots) ERMOD_CUDA(cudaStreamWaitEvent(bst, e.ev_acc[slot], 0));  // slot free again
    ERMOD_CUDA(cudaStreamWaitEvent(bst, e.ev_prep[slot], 0));
    const int half = e.ring_off ? 1 : 0;
    if (e.flush_pend[half]) {  // the first batch in this half waits for its previous flush
      ERMOD_CUDA(cudaStreamWaitEvent(bst, e.ev_flush[half], 0));
      e.flush_pend[half] = false;
    }
    ERMOD_CUDA(cudaMemsetAsync(a.hist, 0, sizeof(int) * (size_t)nb * e.ermax, bst));
    if (e.P.cltype == 0) {
      // bare Coulomb (realcal_bare): no reciprocal space
    } else if (e.mixed) {
      e.phase_begin_on(PH_SPECTRUM, bst);
      ERMOD_CUDA(launch_pme_mixed(e, a));  // spectrum + k3 transform, then (FFT phase) k2/k1
      e.phase_end_on(bst);
    } else {
      e.phase_begin_on(PH_SPECTRUM, bst);
      ERMOD_CUDA(launch_spread64(e, a));
      cufftResult r = cufftExecD2Z(e.plan_d2z, a.phi64, (cufftDoubleComplex*)a.spec64);
      if (r != CUFFT_SUCCESS) return fail_fft(r, "cufftExecD2Z");
      ERMOD_CUDA(launch_influence64(e, a));
      e.phase_end_on(bst);
      e.phase_begin_on(PH_FFT, bst);
      r = cufftExecZ2D(e.plan_z2d, (cufftDoubleComplex*)a.spec64, a.phi64);
      if (r != CUFFT_SUCCESS) return fail_fft(r, "cufftExecZ2D");
      e.phase_end_on(bst);
    }
    e.phase_begin_on(e.mixed ? PH_GATHER : PH_MOL, bst);
    ERMOD_CUDA(launch_mol_energy(e, a));  // mixed: gather, then (mol_energy phase) finish
    e.phase_end_on(bst);
    ERMOD_CUDA(cudaEventRecord(e.ev_done[slot], bst));
    // ---- ordered accumulation on the aux stream ----
    ERMOD_CUDA(cudaStreamWaitEvent(e.aux, e.ev_done[slot], 0));
    e.phase_begin_on(PH_ACCUM, e.aux);
    ERMOD_CUDA(launch_accumulate(e, a, e.aux));
    e.phase_end_on(e.aux);
    if (e.adj_on) {  // after the weights engnmfc of the batch exist
      e.phase_begin_on(PH_ADJOINT, e.aux);
      ERMOD_CUDA(launch_adjoint(e, a, e.aux));
      e.phase_end_on(e.aux);
    }
    ERMOD_CUDA(cudaEventRecord(e.ev_acc[slot], e.aux));
    if (e.P.corrcal) {
      e.ring_fill += nb;
      if (e.ring_fill + B > e.ring_half) {  // flush this half; the next batches fill the other
        // after the half's accumulations (the aux stream runs them in order)
        ERMOD_CUDA(cudaStreamWaitEvent(e.flush, e.ev_acc[slot], 0));
        e.phase_begin_on(PH_ECORR, e.flush);
        ERMOD_CUDA(launch_ecorr_flush(e, e.flush));
        e.phase_end_on(e.flush);
        ERMOD_CUDA(cudaEventRecord(e.ev_flush[half], e.flush));
        e.flush_pend[half] = true;
        e.ring_off = e.ring_half - e.ring_off;
        e.ring_fill = 0;
      }
    } else {
      e.ring_off = e.ring_half - e.ring_off;  // two histogram slots, ordered by ev_acc
    }
  }
  if (e.P.corrcal && e.ring_fill > 0) {
    ERMOD_CUDA(cudaStreamWaitEvent(e.flush, e.ev_acc[(nbatch - 1) % kBatchSlots], 0));
    e.phase_begin_on(PH_ECORR, e.flush);
    ERMOD_CUDA(launch_ecorr_flush(e, e.flush));
    e.phase_end_on(e.flush);
  }
  // the join below orders every flush before the next call's work
  e.ring_fill = 0;
  e.ring_off = 0;
  e.flush_pend[0] = e.flush_pend[1] = false;
  // join every stream back into the caller's stream, then snapshot the status
  // (the flush stream only when ecorr is on: otherwise no work of this call reaches it,
  // and under graph capture it would be a stream outside the capture)
  cudaStream_t others[2 + kBatchStreams] = {e.aux, e.prep};
  for (int k = 0; k < kBatchStreams; ++k) others[2 + k] = e.bs[k];
  const int nj = (dual ? 2 + kBatchStreams : 2);
  for (int k = 0; k < nj + (e.P.corrcal ? 1 : 0); ++k) {
    const cudaStream_t sk = (k < nj) ? others[k] : e.flush;
    ERMOD_CUDA(cudaEventRecord(e.ev_join[k], sk));
    ERMOD_CUDA(cudaStreamWaitEvent(e.stream, e.ev_join[k], 0));
  }
  ERMOD_CUDA(cudaMemcpyAsync(e.h_status, e.d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, e.stream));
  return ERMOD_OK;
}

static int check_ready(Engine& e, int nplace) {
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  if (!e.bins_ready) return fail_param("ermod_set_bins must come first");
  if (!e.frame_ready) return fail_param("ermod_frame must come first");
  if (nplace < 0) return fail_param("nplace < 0");
  return ERMOD_OK;
}

static int reset_status(Engine& e) {  // memsets only, so that a graph capture can hold it
  static_assert(sizeof(DevStatus) == 24, "DevStatus layout: err_key, first_key, mbin_hit, range_fault");
  ERMOD_CUDA(cudaMemsetAsync(&e.d_status->err_key, 0xff, 2 * sizeof(unsigned long long), e.stream));  // kNoError
  ERMOD_CUDA(cudaMemsetAsync(&e.d_status->mbin_hit, 0, 2 * sizeof(int), e.stream));
  *e.h_status = DevStatus{kNoError, kNoError, 0, 0};
  return ERMOD_OK;
}

static int decode_status(Engine& e) {
  const DevStatus s = *e.h_status;
  if (s.mbin_hit || (s.err_key != kNoError && (int)(s.err_key & 0xff) == ERMOD_W_MBIN)) e.warn_bin_firsttime = false;
  if (s.range_fault) {  // the inputs of the batch were out of range: its energies mean nothing
    if (s.range_fault & 4)
      g_err = "non-periodic system: a solute coordinate lies beyond the reach of the frame's fixed-point cube";
    return ERMOD_E_DEVICE;
  }
  // the error of the earliest call wins (device API: later calls stopped at their start)
  const unsigned long long key = (s.first_key != kNoError) ? s.first_key : s.err_key;
  if (key != kNoError) {
    e.err_placement = (int)(key >> 36);
    e.err_molecule = (int)((key >> 8) & 0x0fffffff);
    e.err_energy = std::nan("");
    return (int)(key & 0xff);
  }
  return ERMOD_OK;
}

int ermod_sync(ermod_ctx* c) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  const int st = decode_status(e);
  const int rs = reset_status(e);  // the next calls start a new sequence
  return st ? st : rs;
}

int ermod_placements_device(ermod_ctx* c, int nplace, const int* tag_d, const double* sol_d, const double* sws_d,
                            double* uv_d, double* fl_d) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  int st = check_ready(e, nplace);
  if (st) return st;
  if (nplace == 0) return ERMOD_OK;
  if (!tag_d) return fail_param("tagslt missing");
  // the solute of every placement is the same molecule type in a batch; take its size
  // from the host copy of the topology (tagslt of placement 0 read back)
  int tag0 = 0;
  ERMOD_CUDA(cudaMemcpy(&tag0, tag_d, sizeof(int), cudaMemcpyDeviceToHost));
  if (tag0 < 1 || tag0 > e.nummol) return fail_param("tagslt out of range");
  const int ns = e.numsite[tag0 - 1];
  if (ns > kMaxSoluteSites) {
    g_err = "solute larger than 256 sites";
    return ERMOD_E_UNSUPPORTED;
  }
  // the status stays until ermod_sync: an error of an earlier call stops this one, as
  // the reference stops at the first error
  ERMOD_CUDA(launch_carry_status(e));
  return run_placements(e, nplace, tag_d, sol_d, sws_d, uv_d, fl_d, ns);
}

int ermod_placements(ermod_ctx* c, int nplace, const int* tagslt, const double* sol, const double* sws,
                     double* uv_out, double* fl_out) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  int st = check_ready(e, nplace);
  if (st) return st;
  if (nplace == 0) return ERMOD_OK;
  if (!tagslt) return fail_param("tagslt missing");
  const int ns = e.numsite[std::max(0, std::min(e.nummol - 1, tagslt[0] - 1))];
  for (int p = 0; p < nplace; ++p) {
    if (tagslt[p] < 1 || tagslt[p] > e.nummol) return fail_param("tagslt out of range");
    const int m = tagslt[p] - 1;
    if (e.sluvid[m] == 0) return ERMOD_E_RCP_FST;  // recpcal.F90:468-469
    if (e.numsite[m] > kMaxSoluteSites) {
      g_err = "solute larger than 256 sites";
      return ERMOD_E_UNSUPPORTED;
    }
    if (sol && e.numsite[m] != ns) return fail_param("all placements of a call need the same solute size");
    if (e.P.slttype != 1 && m != e.nummol - 1) {
      g_err = "eng_ins: the inserted solute must be the last molecule";
      return ERMOD_E_PARAM;
    }
  }
  if (e.P.slttype != 1 && !sol) return fail_param("reference mode needs solute_sitepos");
  // uploads
  if (nplace > e.cap_place) {
    dfree(e.d_tagslt);
    dfree(e.d_solxyz);
    dfree(e.d_sws);
    e.cap_place = std::max(nplace, 1024);
    ERMOD_CUDA(dalloc(&e.d_tagslt, e.cap_place));
    ERMOD_CUDA(dalloc(&e.d_solxyz, (size_t)e.cap_place * kMaxSoluteSites * 3));
    ERMOD_CUDA(dalloc(&e.d_sws, e.cap_place));
  }
  e.phase_begin(PH_COPY);
  ERMOD_CUDA(cudaMemcpyAsync(e.d_tagslt, tagslt, sizeof(int) * nplace, cudaMemcpyHostToDevice, e.stream));
  if (sol)
    ERMOD_CUDA(cudaMemcpyAsync(e.d_solxyz, sol, sizeof(double) * 3 * (size_t)ns * nplace, cudaMemcpyHostToDevice,
                               e.stream));
  if (sws) ERMOD_CUDA(cudaMemcpyAsync(e.d_sws, sws, sizeof(double) * nplace, cudaMemcpyHostToDevice, e.stream));
  e.phase_end();
  double* d_uv = nullptr;
  double* d_fl = nullptr;
  if (uv_out) ERMOD_CUDA(dalloc(&d_uv, (size_t)nplace * (e.slvmax + 1)));
  if (fl_out) ERMOD_CUDA(dalloc(&d_fl, (size_t)nplace * e.numslv));
  st = reset_status(e);
  if (!st) st = run_placements(e, nplace, e.d_tagslt, sol ? e.d_solxyz : nullptr, sws ? e.d_sws : nullptr, d_uv, d_fl, ns);
  if (!st) {
    if (uv_out)
      st = cudaMemcpyAsync(uv_out, d_uv, sizeof(double) * (size_t)nplace * (e.slvmax + 1), cudaMemcpyDeviceToHost,
                           e.stream) == cudaSuccess ? ERMOD_OK : ERMOD_E_CUDA;
    if (fl_out && !st)
      st = cudaMemcpyAsync(fl_out, d_fl, sizeof(double) * (size_t)nplace * e.numslv, cudaMemcpyDeviceToHost,
                           e.stream) == cudaSuccess ? ERMOD_OK : ERMOD_E_CUDA;
  }
  const int st2 = ermod_sync(c);
  if (d_uv) cudaFree(d_uv);
  if (d_fl) cudaFree(d_fl);
  return st ? st : st2;
}

int ermod_clear(ermod_ctx* c) {  // engclear (engproc.F90:276-288)
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  if (!e.bins_ready) return fail_param("ermod_set_bins must come first");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaMemsetAsync(e.d_edens, 0, sizeof(double) * e.ermax, e.stream));
  if (e.d_ecorr) ERMOD_CUDA(cudaMemsetAsync(e.d_ecorr, 0, sizeof(double) * (size_t)e.ermax * e.ermax, e.stream));
  if (e.d_ecorr_n)
    ERMOD_CUDA(cudaMemsetAsync(e.d_ecorr_n, 0, sizeof(long long) * (size_t)e.ermax * e.ermax, e.stream));
  ERMOD_CUDA(cudaMemsetAsync(e.d_eself, 0, sizeof(double) * std::max(e.esmax, 1), e.stream));
  ERMOD_CUDA(cudaMemsetAsync(e.d_slnuv, 0, sizeof(double) * e.numslv, e.stream));
  ERMOD_CUDA(cudaMemsetAsync(e.d_scal, 0, sizeof(double) * 3, e.stream));  // engnorm, engsmpl, avslf
  if (e.d_edintm)  // engclear's hunk of the intermediate-state extension
    ERMOD_CUDA(cudaMemsetAsync(e.d_edintm, 0, sizeof(double) * ((size_t)e.ermax + e.numslv + 3), e.stream));
  if (e.adj_on) {
    ERMOD_CUDA(cudaMemsetAsync(e.d_adj_grad, 0, sizeof(double) * 3 * (size_t)e.adj_ns * e.ermax, e.stream));
    ERMOD_CUDA(cudaMemsetAsync(e.d_adj_w, 0, sizeof(double) * e.ermax, e.stream));
  }
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  return ERMOD_OK;
}

static void free_intermediate(Engine& e) {
  dfree(e.d_int_mask);
  dfree(e.d_edintm);
}

static void free_config_check(Engine& e) {
  dfree(e.d_agg_mass);
  dfree(e.d_site_mass);
  dfree(e.d_ref_atoms);
  dfree(e.d_ref_host);
  dfree(e.d_ref_slt);
  dfree(e.d_ref_fit);
  dfree(e.d_skip);
  e.cap_skip = 0;
  e.ref_nh = e.ref_ns = 0;
  e.cfg_pos = e.cfg_str = 0;
}

static void free_library(Engine& e) {
  dfree(e.d_lib);
  dfree(e.d_lib_wt);
  dfree(e.d_lib_acc);
  e.lib_nconf = e.lib_ns = e.lib_nwt = e.lib_na = 0;
}

// getsolute (insertion.F90:384-495) for the device generator: the structure library, its
// weights and the structures that pass insstructure's window, in file order
int ermod_set_solute_library(ermod_ctx* c, int nconf, int nsite, const double* conf, int nweight,
                             const double* weight, int insstructure, double lwstr, double upstr) {
  if (!c) return fail_param("null argument");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  if (nconf == 0) {
    free_library(e);
    return ERMOD_OK;
  }
  if (nconf < 0 || !conf) return fail_param("nconf must be >= 0 and conf not NULL");
  if (nsite < 1 || nsite > kMaxSoluteSites) return fail_param("nsite must be 1..256");
  if (nweight < 0 || (nweight > 0 && !weight)) return fail_param("nweight must be >= 0, weight not NULL");
  if (insstructure != 0 && insstructure != 1) return fail_param("insstructure 0 or 1");
  if (insstructure == 1) {
    if (e.ref_ns == 0) return fail_param("insstructure 1 needs ermod_set_reference_structure");
    if (nsite != e.ref_ns) {  // size(psite) /= size(refslt_crd) (insertion.F90:463-464)
      g_err = "ins_siz: the library's structures and the reference solute differ in size";
      return ERMOD_E_INS_SIZ;
    }
  }
  free_library(e);
  const int nwt = (weight && nweight > 0) ? nweight : 0;
  ERMOD_CUDA(dalloc(&e.d_lib, 3 * (size_t)nsite * nconf));
  ERMOD_CUDA(dalloc(&e.d_lib_wt, (size_t)std::max(nwt, 1)));
  ERMOD_CUDA(dalloc(&e.d_lib_acc, (size_t)nconf + 1));
  ERMOD_CUDA(cudaMemcpy(e.d_lib, conf, sizeof(double) * 3 * nsite * (size_t)nconf, cudaMemcpyHostToDevice));
  if (nwt) ERMOD_CUDA(cudaMemcpy(e.d_lib_wt, weight, sizeof(double) * nwt, cudaMemcpyHostToDevice));
  e.lib_nconf = nconf;
  e.lib_ns = nsite;
  e.lib_nwt = nwt;
  ERMOD_CUDA(launch_library_filter(e, insstructure, lwstr, upstr));
  int na = 0;
  ERMOD_CUDA(cudaMemcpyAsync(&na, e.d_lib_acc + nconf, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  if (na <= 0) {
    free_library(e);
    return fail_param("no structure of the library lies in [lwstr, upstr] (getsolute would read forever)");
  }
  e.lib_na = na;
  return ERMOD_OK;
}

// hostspec's aggregate and the site masses (com_aggregate, insertion.F90:539-566)
int ermod_set_aggregate(ermod_ctx* c, const int* host_mol, const double* sitemass) {
  if (!c || !host_mol || !sitemass) return fail_param("null argument");
  Engine& e = c->e;
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  std::vector<double> hm((size_t)e.numatm, 0.0);
  double tot = 0.0;
  for (int i = 0; i < e.nummol; ++i)
    if (host_mol[i])
      for (int a = e.mbi0[i]; a < e.mbi0[i + 1]; ++a) {
        hm[a] = sitemass[a];
        tot += sitemass[a];
      }
  if (!(tot > 0.0)) return fail_param("bst_zrw: the host aggregate has no mass");
  for (int i = 0; i < e.nummol; ++i) {  // center_of_mass of a solute (bestfit.F90:167-168)
    if (e.sluvid[i] == 0) continue;
    double m = 0.0;
    for (int a = e.mbi0[i]; a < e.mbi0[i + 1]; ++a) m += sitemass[a];
    if (m == 0.0) return fail_param("bst_zrw: a solute molecule has no mass");
  }
  if (!e.d_agg_mass) ERMOD_CUDA(dalloc(&e.d_agg_mass, (size_t)e.numatm));
  if (!e.d_site_mass) ERMOD_CUDA(dalloc(&e.d_site_mass, (size_t)e.numatm));
  ERMOD_CUDA(cudaMemcpy(e.d_agg_mass, hm.data(), sizeof(double) * e.numatm, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_site_mass, sitemass, sizeof(double) * e.numatm, cudaMemcpyHostToDevice));
  return ERMOD_OK;
}

// load_refstructure (insertion.F90:619-700): refspec atoms and the reference solute
int ermod_set_reference_structure(ermod_ctx* c, const int* ref_mol, const double* refhost_crd,
                                  const double* refhost_weight, int refslt_natom, const double* refslt_crd,
                                  const double* refslt_weight) {
  if (!c || !ref_mol || !refslt_crd || !refslt_weight) return fail_param("null argument");
  Engine& e = c->e;
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  if (refslt_natom <= 0 || refslt_natom > kMaxSoluteSites) return fail_param("refslt_natom out of range");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  std::vector<int> atoms;
  for (int i = 0; i < e.nummol; ++i)
    if (ref_mol[i])
      for (int a = e.mbi0[i]; a < e.mbi0[i + 1]; ++a) atoms.push_back(a);
  const int nh = (int)atoms.size();
  if (nh > 0 && (!refhost_crd || !refhost_weight)) return fail_param("null reference host");
  std::vector<double> host(4 * (size_t)std::max(nh, 1)), slt(4 * (size_t)refslt_natom);
  double wh = 0.0, ws = 0.0;
  for (int k = 0; k < nh; ++k) {
    for (int i = 0; i < 3; ++i) host[4 * k + i] = refhost_crd[3 * k + i];
    host[4 * k + 3] = refhost_weight[k];
    wh += refhost_weight[k];
  }
  for (int k = 0; k < refslt_natom; ++k) {
    for (int i = 0; i < 3; ++i) slt[4 * k + i] = refslt_crd[3 * k + i];
    slt[4 * k + 3] = refslt_weight[k];
    ws += refslt_weight[k];
  }
  if (nh > 0 && wh == 0.0) return fail_param("bst_zrw: the reference host has no weight");
  if (ws == 0.0) return fail_param("bst_zrw: the reference solute has no weight");
  dfree(e.d_ref_atoms);
  dfree(e.d_ref_host);
  dfree(e.d_ref_slt);
  ERMOD_CUDA(dalloc(&e.d_ref_atoms, (size_t)std::max(nh, 1)));
  ERMOD_CUDA(dalloc(&e.d_ref_host, host.size()));
  ERMOD_CUDA(dalloc(&e.d_ref_slt, slt.size()));
  if (nh > 0) ERMOD_CUDA(cudaMemcpy(e.d_ref_atoms, atoms.data(), sizeof(int) * nh, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_ref_host, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemcpy(e.d_ref_slt, slt.data(), sizeof(double) * slt.size(), cudaMemcpyHostToDevice));
  e.ref_nh = nh;
  e.ref_ns = refslt_natom;
  return ERMOD_OK;
}

// check_mol_configuration (engproc.F90:1046-1100): solution mode
int ermod_set_configuration_check(ermod_ctx* c, int insposition, double lwreg, double upreg, int insstructure,
                                  double lwstr, double upstr) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  if (insposition < 0 || insposition > 6 || insstructure < 0 || insstructure > 1)
    return fail_param("insposition 0..6, insstructure 0..1");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  const int pos = (insposition >= 2 && insposition <= 5) ? insposition : 0;  // 0, 1, 6 test nothing
  if ((pos == 3 || pos == 4) && e.P.boxshp == 0) {
    g_err = "eng_slb: a slab check needs a periodic system";
    return ERMOD_E_ENG_SLB;
  }
  if (pos >= 2 && pos <= 4 && !e.d_agg_mass) return fail_param("ermod_set_aggregate must come first");
  if (pos == 5 || insstructure == 1) {
    if (e.ref_ns == 0) return fail_param("ermod_set_reference_structure must come first");
    if (pos == 5 && e.ref_nh == 0) return fail_param("insposition 5 needs reference host atoms");
    for (int i = 0; i < e.nummol; ++i)  // numsite(tagslt) /= refslt_natom stops the reference
      if (e.sluvid[i] == 1 && e.mbi0[i + 1] - e.mbi0[i] != e.ref_ns)
        return fail_param("eng_bug: a solute molecule and the reference solute differ in size");
  }
  e.cfg_pos = pos;
  e.cfg_str = insstructure;
  e.cfg_lw = lwreg;
  e.cfg_up = upreg;
  e.cfg_lwstr = lwstr;
  e.cfg_upstr = upstr;
  if ((pos || insstructure) && e.cap_skip < std::max(64, e.nummol)) {
    dfree(e.d_skip);
    e.cap_skip = std::max(64, e.nummol);
    ERMOD_CUDA(dalloc(&e.d_skip, (size_t)e.cap_skip));
  }
  return ERMOD_OK;
}

int ermod_intermediate_enable(ermod_ctx* c, const double* refs_density) {
  if (!c || !refs_density) return fail_param("null argument");
  Engine& e = c->e;
  if (!e.bins_ready) return fail_param("ermod_set_bins must come first");
  if (e.P.slttype != 1) return fail_param("the intermediate state applies to solution mode only");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  free_intermediate(e);
  std::vector<unsigned char> mask(e.ermax);
  for (int i = 0; i < e.ermax; ++i) mask[i] = (refs_density[i] > 1.0e-30) ? 0 : 1;  // tiny, engproc.F90:23
  ERMOD_CUDA(dalloc(&e.d_int_mask, (size_t)e.ermax));
  ERMOD_CUDA(dalloc(&e.d_edintm, (size_t)e.ermax + e.numslv + 3));
  ERMOD_CUDA(cudaMemcpy(e.d_int_mask, mask.data(), e.ermax, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemset(e.d_edintm, 0, sizeof(double) * ((size_t)e.ermax + e.numslv + 3)));
  return ERMOD_OK;
}

int ermod_intermediate_get(ermod_ctx* c, double* edintm, double* uvintm, double* totals) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  if (!e.d_edintm) return fail_param("ermod_intermediate_enable must come first");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  std::vector<double> h((size_t)e.ermax + e.numslv + 3);
  ERMOD_CUDA(cudaMemcpy(h.data(), e.d_edintm, sizeof(double) * h.size(), cudaMemcpyDeviceToHost));
  if (edintm) std::copy(h.begin(), h.begin() + e.ermax, edintm);
  if (uvintm) std::copy(h.begin() + e.ermax, h.begin() + e.ermax + e.numslv, uvintm);
  if (totals) std::copy(h.begin() + e.ermax + e.numslv, h.end(), totals);
  return ERMOD_OK;
}

static void free_adjoint(Engine& e) {
  dfree(e.d_adj_grad);
  dfree(e.d_adj_w);
  dfree(e.d_adj_par);
  dfree(e.d_adj_du);
  dfree(e.d_adj_key);
  dfree(e.d_adj_seg);
  if (e.d_adj_cub) cudaFree(e.d_adj_cub);
  e.d_adj_cub = nullptr;
  dfree(e.d_mol_bin);
  dfree(e.d_ps_nsite);
  dfree(e.d_ps_qf);
  dfree(e.d_ps_bvec);
  dfree(e.d_ps_self);
  e.adj_on = false;
}

int ermod_adjoint_enable(ermod_ctx* c, int solute_mol, int cmbrule) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  if (!e.mixed || e.P.cltype == 0) {
    g_err = "the adjoint runs on the mixed-precision PME/PPPM path only";
    return ERMOD_E_UNSUPPORTED;
  }
  if (!e.topo_ready) return fail_param("ermod_set_topology must come first");
  if (!e.bins_ready) return fail_param("ermod_set_bins must come first");
  if (solute_mol < 1 || solute_mol > e.nummol) return fail_param("solute_mol out of range");
  if (cmbrule < 0 || cmbrule > 1) return fail_param("cmbrule must be 0 or 1");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  free_adjoint(e);
  const int ns = e.numsite[solute_mol - 1];
  if (ns < 1 || ns > kMaxSoluteSites) return fail_param("the solute has no sites or too many");
  int st = ensure_batch(e);
  if (st) return st;
  const int T = e.ljtype_max;
  std::vector<double> lje((size_t)T * T), ljl((size_t)T * T);
  ERMOD_CUDA(cudaMemcpy(lje.data(), e.d_ljene, sizeof(double) * lje.size(), cudaMemcpyDeviceToHost));
  ERMOD_CUDA(cudaMemcpy(ljl.data(), e.d_ljlensq, sizeof(double) * ljl.size(), cudaMemcpyDeviceToHost));
  std::vector<float2> par(ns);
  for (int s = 0; s < ns; ++s) {  // eps_s = ljene(t,t), sigma_s^2 = ljlensq(t,t) under either rule
    const int t = e.ljtype0[e.mbi0[solute_mol - 1] + s];
    par[s] = make_float2((float)lje[(size_t)t * T + t], (float)std::sqrt(ljl[(size_t)t * T + t]));
  }
  const int B = e.Bmax;
  ERMOD_CUDA(dalloc(&e.d_adj_grad, 3 * (size_t)ns * e.ermax));
  ERMOD_CUDA(dalloc(&e.d_adj_w, (size_t)e.ermax));
  ERMOD_CUDA(dalloc(&e.d_adj_par, (size_t)ns));
  ERMOD_CUDA(dalloc(&e.d_adj_du, (size_t)e.slvmax * 3 * ns));
  ERMOD_CUDA(dalloc(&e.d_adj_key, 4 * (size_t)e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_adj_seg, 2 * (size_t)e.ermax));
  e.adj_cub_bytes = adjoint_cub_bytes(e.slvmax);
  ERMOD_CUDA(cudaMalloc(&e.d_adj_cub, std::max<size_t>(e.adj_cub_bytes, 16)));
  ERMOD_CUDA(dalloc(&e.d_mol_bin, (size_t)kBatchSlots * B * e.slvmax));
  ERMOD_CUDA(dalloc(&e.d_ps_nsite, (size_t)B));
  ERMOD_CUDA(dalloc(&e.d_ps_qf, (size_t)B * kMaxSoluteSites));
  ERMOD_CUDA(dalloc(&e.d_ps_bvec, (size_t)B * kMaxSoluteSites * 3 * e.Kmax()));
  ERMOD_CUDA(dalloc(&e.d_ps_self, (size_t)B * spectrum_partials(e)));
  ERMOD_CUDA(cudaMemcpy(e.d_adj_par, par.data(), sizeof(float2) * ns, cudaMemcpyHostToDevice));
  ERMOD_CUDA(cudaMemset(e.d_adj_grad, 0, sizeof(double) * 3 * (size_t)ns * e.ermax));
  ERMOD_CUDA(cudaMemset(e.d_adj_w, 0, sizeof(double) * e.ermax));
  ERMOD_CUDA(cudaMemset(e.d_ps_qf, 0, sizeof(float) * (size_t)B * kMaxSoluteSites));
  e.adj_mol = solute_mol;
  e.adj_ns = ns;
  e.adj_cmbrule = cmbrule;
  e.adj_on = true;
  return ERMOD_OK;
}

int ermod_adjoint_get(ermod_ctx* c, double* grad, double* weight, int* nparam) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  if (!e.adj_on) return fail_param("ermod_adjoint_enable must come first");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  if (nparam) *nparam = 3 * e.adj_ns;
  if (grad)
    ERMOD_CUDA(cudaMemcpy(grad, e.d_adj_grad, sizeof(double) * 3 * (size_t)e.adj_ns * e.ermax,
                          cudaMemcpyDeviceToHost));
  if (weight) ERMOD_CUDA(cudaMemcpy(weight, e.d_adj_w, sizeof(double) * e.ermax, cudaMemcpyDeviceToHost));
  return ERMOD_OK;
}

int ermod_get_accum(ermod_ctx* c, double* edens, double* ecorr, double* eself, double* slnuv, double* minuv,
                    double* maxuv, double* scalars, int64_t* ecorr_count) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  if (!e.bins_ready) return fail_param("ermod_set_bins must come first");
  cudaSetDevice(e.device);
  ERMOD_CUDA(cudaStreamSynchronize(e.stream));
  const size_t E = e.ermax;
  if (edens) ERMOD_CUDA(cudaMemcpy(edens, e.d_edens, sizeof(double) * E, cudaMemcpyDeviceToHost));
  if (ecorr) {
    if (!e.d_ecorr) return fail_param("corrcal is off");
    ERMOD_CUDA(cudaMemcpy(ecorr, e.d_ecorr, sizeof(double) * E * E, cudaMemcpyDeviceToHost));
  }
  if (ecorr_count) {
    if (!e.d_ecorr_n) return fail_param("count_mirror is off");
    ERMOD_CUDA(cudaMemcpy(ecorr_count, e.d_ecorr_n, sizeof(long long) * E * E, cudaMemcpyDeviceToHost));
  }
  if (eself && e.esmax > 0) ERMOD_CUDA(cudaMemcpy(eself, e.d_eself, sizeof(double) * e.esmax, cudaMemcpyDeviceToHost));
  if (slnuv) ERMOD_CUDA(cudaMemcpy(slnuv, e.d_slnuv, sizeof(double) * e.numslv, cudaMemcpyDeviceToHost));
  if (minuv) ERMOD_CUDA(cudaMemcpy(minuv, e.d_minuv, sizeof(double) * (e.numslv + 1), cudaMemcpyDeviceToHost));
  if (maxuv) ERMOD_CUDA(cudaMemcpy(maxuv, e.d_maxuv, sizeof(double) * (e.numslv + 1), cudaMemcpyDeviceToHost));
  if (scalars) {
    double s[8];
    ERMOD_CUDA(cudaMemcpy(s, e.d_scal, sizeof(s), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 5; ++i) scalars[i] = s[i];
  }
  return ERMOD_OK;
}

int ermod_get_sizes(const ermod_ctx* c, int* slvmax, int* ermax, int* esmax, int* numslv) {
  if (!c) return fail_param("null context");
  if (slvmax) *slvmax = c->e.slvmax;
  if (ermax) *ermax = c->e.ermax;
  if (esmax) *esmax = c->e.esmax;
  if (numslv) *numslv = c->e.numslv;
  return ERMOD_OK;
}

int ermod_error_info(const ermod_ctx* c, int* placement, int* molecule, double* energy) {
  if (!c) return fail_param("null context");
  if (placement) *placement = c->e.err_placement;
  if (molecule) *molecule = c->e.err_molecule;
  if (energy) *energy = c->e.err_energy;
  return ERMOD_OK;
}

int ermod_timing_enable(ermod_ctx* c, int on) {
  if (!c) return fail_param("null context");
  c->e.timing = on != 0;
  return ERMOD_OK;
}

int ermod_timing_reset(ermod_ctx* c) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  harvest(e);
  for (double& v : e.phase_ms) v = 0.0;
  e.launches = 0;
  return ERMOD_OK;
}

int ermod_timing_get(ermod_ctx* c, int max_phases, double* ms, const char** names, int* nphases, int64_t* launches) {
  if (!c) return fail_param("null context");
  Engine& e = c->e;
  cudaSetDevice(e.device);
  harvest(e);
  const int n = std::min(max_phases, (int)PH_COUNT);
  for (int i = 0; i < n; ++i) {
    if (ms) ms[i] = e.phase_ms[i];
    if (names) names[i] = kPhaseNames[i];
  }
  if (nphases) *nphases = PH_COUNT;
  if (launches) *launches = e.launches;
  return ERMOD_OK;
}

int ermod_ecorr_add_noalloc(const int* hist, const double* weight, int nplace, int ermax, double* ecorr,
                            int64_t* ecorr_count, void* stream) {
  if (nplace < 0 || ermax < 1) return fail_param("ermod_ecorr_add_noalloc: nplace >= 0 and ermax >= 1 required");
  if (nplace > kNoAllocMaxPlace || ermax > kNoAllocMaxBins || (long long)nplace * ermax > kNoAllocMaxEntries) {
    set_error_string("ermod_ecorr_add_noalloc: nplace = " + std::to_string(nplace) + ", ermax = " +
                     std::to_string(ermax) + " exceed its fixed scratch (nplace <= " +
                     std::to_string(kNoAllocMaxPlace) + ", ermax <= " + std::to_string(kNoAllocMaxBins) +
                     ", nplace * ermax <= " + std::to_string(kNoAllocMaxEntries) + ")");
    return ERMOD_E_PARAM;
  }
  if (nplace == 0) return ERMOD_OK;
  if (!hist || !weight || !ecorr) return fail_param("ermod_ecorr_add_noalloc: null hist, weight or ecorr");
  const cudaError_t err = launch_ecorr_noalloc(hist, weight, nplace, ermax, ecorr, (long long*)ecorr_count,
                                               (cudaStream_t)stream);
  if (err != cudaSuccess) return fail_cuda(err, "ermod_ecorr_add_noalloc");
  return ERMOD_OK;
}

int ermod_generate_placements(ermod_ctx* c, int nplace, int nsite, const double* bfcoord, const double* mass,
                              const ermod_insert_params* ip, double* sol_d, double* sws_d) {
  if (!c || !mass || !ip || (nplace > 0 && !sol_d)) return fail_param("null argument");
  Engine& e = c->e;
  const bool lib = e.lib_nconf > 0;  // structures from the library (bfcoord unused)
  if (!lib && !bfcoord) return fail_param("null bfcoord");
  if (!e.frame_ready) return fail_param("ermod_frame must come first (its cell is used)");
  if (nsite < 1 || nsite > kMaxSoluteSites) return fail_param("nsite must be 1..256");
  if (lib && nsite != e.lib_ns) {  // size(psite) /= size(bfcoord) (insertion.F90:440)
    g_err = "ins_siz: the library's structures and the solute differ in size";
    return ERMOD_E_INS_SIZ;
  }
  if (ip->insposition < 0 || ip->insposition > 6 || ip->insorient < 0 || ip->insorient > 1 || ip->insorigin < 0 ||
      ip->insorigin > 3)
    return fail_param("insposition 0..6, insorient 0..1, insorigin 0..3");
  if (ip->insorigin == 2 && !e.d_agg_mass) return fail_param("insorigin 2 needs ermod_set_aggregate");
  if (ip->insorigin == 3) {
    if (e.ref_ns == 0 || e.ref_nh == 0) return fail_param("insorigin 3 needs ermod_set_reference_structure");
    if (nsite != e.ref_ns) return fail_param("ins_bug: the solute and the reference solute differ in size");
    // check_solute_configuration accepts only these with the reference structure
    if (ip->insposition != 5 && ip->insposition != 6) return fail_param("ins_bug: insorigin 3 needs insposition 5 or 6");
  }
  if ((ip->insposition == 2 || ip->insposition == 3 || ip->insposition == 4) && !(ip->upreg >= ip->lwreg))
    return fail_param("upreg < lwreg");
  if ((ip->insposition == 5 || ip->insposition == 6) && !(ip->upreg > 0.0)) return fail_param("upreg must be > 0");
  if (e.P.boxshp == 0 && (ip->insposition == 0 || ip->insposition == 3 || ip->insposition == 4)) {
    g_err = "ins_geo: random and slab insertion need a periodic system";  // insertion.F90:155,186
    return ERMOD_E_INS_GEO;
  }
  if (nplace <= 0) return ERMOD_OK;
  cudaSetDevice(e.device);
  if (!e.d_ins) ERMOD_CUDA(dalloc(&e.d_ins, 4 * (size_t)kMaxSoluteSites));
  if (ip->insorigin >= 2 && !e.d_ref_fit) ERMOD_CUDA(dalloc(&e.d_ref_fit, 6 * (size_t)kMaxSoluteSites + 8));
  if (lib)  // the origin kernel's rigid starting structure is unused; give it the first one
    ERMOD_CUDA(cudaMemcpyAsync(e.d_ins, e.d_lib, sizeof(double) * 3 * nsite, cudaMemcpyDeviceToDevice, e.stream));
  else
    ERMOD_CUDA(cudaMemcpyAsync(e.d_ins, bfcoord, sizeof(double) * 3 * nsite, cudaMemcpyHostToDevice, e.stream));
  ERMOD_CUDA(cudaMemcpyAsync(e.d_ins + 3 * kMaxSoluteSites, mass, sizeof(double) * nsite, cudaMemcpyHostToDevice,
                             e.stream));
  ERMOD_CUDA(launch_insert(e, nplace, nsite, *ip, e.d_ins, e.d_ins + 3 * kMaxSoluteSites, sol_d, sws_d));
  return ERMOD_OK;
}

// ---- several systems in one CUDA graph --------------------------------------------
struct ermod_graph {
  int device = 0;
  std::vector<ermod_ctx*> ctx;
  std::vector<cudaStream_t> fork;  // one capture stream per system
  cudaStream_t origin = nullptr;
  cudaEvent_t ev_fork = nullptr;
  std::vector<cudaEvent_t> ev_sys;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t launched = nullptr;
};

int ermod_graph_destroy(ermod_graph* g) {
  if (!g) return ERMOD_OK;
  cudaSetDevice(g->device);
  if (g->exec) cudaStreamSynchronize(g->launched);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (cudaEvent_t ev : g->ev_sys)
    if (ev) cudaEventDestroy(ev);
  if (g->ev_fork) cudaEventDestroy(g->ev_fork);
  for (cudaStream_t st : g->fork)
    if (st) cudaStreamDestroy(st);
  if (g->origin) cudaStreamDestroy(g->origin);
  delete g;
  return ERMOD_OK;
}

int ermod_graph_create(int nctx, ermod_ctx* const* ctx, const double* const* sitepos_d, const double* cells,
                       const double* stat_weight_system, const int* nplace, const int* solute_mol,
                       const int* const* tag_d, const double* const* sol_d, const double* const* sws_d,
                       ermod_graph** out) {
  if (!out || nctx <= 0 || !ctx || !sitepos_d || !cells || !nplace || !solute_mol || !tag_d)
    return fail_param("null argument or no systems");
  *out = nullptr;
  const int device = ctx[0] ? ctx[0]->e.device : 0;
  for (int i = 0; i < nctx; ++i) {
    if (!ctx[i] || !sitepos_d[i] || (nplace[i] > 0 && !tag_d[i])) return fail_param("null context or input");
    Engine& e = ctx[i]->e;
    if (e.device != device) return fail_param("all systems of a graph need the same device");
    if (!e.mixed) {
      g_err = "graph capture runs the mixed-precision path only";
      return ERMOD_E_UNSUPPORTED;
    }
    if (e.P.boxshp == 0) {  // its frame set-up reads the coordinate extent back to the host
      g_err = "graph capture takes periodic systems only";
      return ERMOD_E_UNSUPPORTED;
    }
    if (!e.topo_ready || !e.bins_ready || !e.frame_ready || !e.buf.u_nsite)
      return fail_param("every system needs one ordinary frame + placements step before capture");
    if (solute_mol[i] < 1 || solute_mol[i] > e.nummol) return fail_param("solute_mol out of range");
    if (e.numsite[solute_mol[i] - 1] > kMaxSoluteSites) {
      g_err = "solute larger than 256 sites";
      return ERMOD_E_UNSUPPORTED;
    }
    if (e.P.slttype != 1 && nplace[i] > 0 && !(sol_d && sol_d[i]))
      return fail_param("reference mode needs solute_sitepos");
  }
  cudaSetDevice(device);
  ermod_graph* g = new ermod_graph();
  g->device = device;
  g->ctx.assign(ctx, ctx + nctx);
  g->fork.assign(nctx, nullptr);
  g->ev_sys.assign(nctx, nullptr);
  cudaError_t err;
#define ERMOD_G(call)                        \
  do {                                       \
    if ((err = (call)) != cudaSuccess) {     \
      const int st_ = fail_cuda(err, #call); \
      ermod_graph_destroy(g);                \
      return st_;                            \
    }                                        \
  } while (0)
  ERMOD_G(cudaStreamCreateWithFlags(&g->origin, cudaStreamNonBlocking));
  ERMOD_G(cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming));
  for (int i = 0; i < nctx; ++i) {
    ERMOD_G(cudaStreamCreateWithFlags(&g->fork[i], cudaStreamNonBlocking));
    ERMOD_G(cudaEventCreateWithFlags(&g->ev_sys[i], cudaEventDisableTiming));
  }
  // every context finishes its queued work before its streams join the capture
  for (int i = 0; i < nctx; ++i) ERMOD_G(cudaStreamSynchronize(ctx[i]->e.stream));
  ERMOD_G(cudaStreamBeginCapture(g->origin, cudaStreamCaptureModeThreadLocal));
  int st = ERMOD_OK;
  if ((err = cudaEventRecord(g->ev_fork, g->origin)) != cudaSuccess) st = fail_cuda(err, "fork");
  for (int i = 0; i < nctx && st == ERMOD_OK; ++i) {
    Engine& e = ctx[i]->e;
    const cudaStream_t saved = e.stream;
    const bool saved_timing = e.timing;
    e.stream = g->fork[i];
    e.timing = false;
    if ((err = cudaStreamWaitEvent(e.stream, g->ev_fork, 0)) != cudaSuccess) st = fail_cuda(err, "fork");
    if (st == ERMOD_OK)
      st = frame_common(e, cells + 9 * (size_t)i, stat_weight_system ? stat_weight_system[i] : 1.0, 0.0);
    if (st == ERMOD_OK &&
        (err = cudaMemcpyAsync(e.d_sitepos, sitepos_d[i], sizeof(double) * 3 * e.numatm, cudaMemcpyDeviceToDevice,
                               e.stream)) != cudaSuccess)
      st = fail_cuda(err, "frame copy");
    if (st == ERMOD_OK) st = frame_launch(e);
    if (st == ERMOD_OK && nplace[i] > 0) st = reset_status(e);
    if (st == ERMOD_OK && nplace[i] > 0)
      st = run_placements(e, nplace[i], tag_d[i], sol_d ? sol_d[i] : nullptr, sws_d ? sws_d[i] : nullptr, nullptr,
                          nullptr, e.numsite[solute_mol[i] - 1]);
    if (st == ERMOD_OK && (err = cudaEventRecord(g->ev_sys[i], e.stream)) != cudaSuccess) st = fail_cuda(err, "join");
    if (st == ERMOD_OK && (err = cudaStreamWaitEvent(g->origin, g->ev_sys[i], 0)) != cudaSuccess)
      st = fail_cuda(err, "join");
    e.stream = saved;
    e.timing = saved_timing;
  }
  cudaGraph_t graph = nullptr;
  err = cudaStreamEndCapture(g->origin, &graph);
  g->graph = graph;
  if (st != ERMOD_OK) {
    ermod_graph_destroy(g);
    return st;
  }
  ERMOD_G(err);
  ERMOD_G(cudaGraphInstantiate(&g->exec, g->graph, 0));
#undef ERMOD_G
  *out = g;
  return ERMOD_OK;
}

int ermod_graph_launch(ermod_graph* g, void* stream) {
  if (!g || !g->exec) return fail_param("null graph");
  cudaSetDevice(g->device);
  g->launched = (cudaStream_t)stream;
  ERMOD_CUDA(cudaGraphLaunch(g->exec, g->launched));
  return ERMOD_OK;
}

int ermod_graph_sync(ermod_graph* g) {
  if (!g) return fail_param("null graph");
  cudaSetDevice(g->device);
  ERMOD_CUDA(cudaStreamSynchronize(g->launched));
  int first = ERMOD_OK;
  for (ermod_ctx* c : g->ctx) {
    const int st = decode_status(c->e);
    if (st != ERMOD_OK && first == ERMOD_OK) first = st;
  }
  return first;
}

}  // extern "C"
