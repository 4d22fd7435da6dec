// Host side of the G-MCTDH propagation core: plans the batched kernels for one
// model once (mctdh_create), then runs the equation of motion, the adaptive
// Runge-Kutta steps, the CMF2 steps and the observables on device-resident
// state.  The C-ABI it exports is declared in include/macaw_gb300.h.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/macaw_gb300.h"
#include "kernels.cuh"

namespace {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};
struct StatusError : std::runtime_error {
  int64_t code;
  StatusError(int64_t c, const std::string& s) : std::runtime_error(s), code(c) {}
};

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess)                                                                        \
      throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_) + " at " __FILE__ ":" + \
                      std::to_string(__LINE__));                                                  \
  } while (0)

std::string g_create_error;

// Bump allocator over large device chunks; buffers live as long as the context.
struct DevArena {
  std::vector<void*> chunks;
  char* cur = nullptr;
  size_t left = 0;
  size_t total = 0;
  size_t chunk = (size_t)64 << 20;   // smallest cudaMalloc
  void* alloc(size_t bytes) {
    bytes = (bytes + 255) & ~(size_t)255;
    if (bytes == 0) bytes = 256;
    if (bytes > left) {
      size_t sz = std::max(bytes, chunk);
      void* p = nullptr;
      CK(cudaMalloc(&p, sz));
      chunks.push_back(p);
      cur = (char*)p;
      left = sz;
      total += sz;
    }
    void* r = cur;
    cur += bytes;
    left -= bytes;
    return r;
  }
  cplx* calloc_c(long long n) { return (cplx*)alloc(sizeof(cplx) * (size_t)std::max(n, 1LL)); }
  ~DevArena() {
    for (void* p : chunks) cudaFree(p);
  }
};

template <typename T>
T* upload_vec(DevArena& ar, const std::vector<T>& v) {
  if (v.empty()) return nullptr;
  T* d = (T*)ar.alloc(sizeof(T) * v.size());
  CK(cudaMemcpy(d, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  return d;
}

// A tensor view: device pointer + per-mode sizes (mode 1 fastest).
struct TRef {
  cplx* p = nullptr;
  std::vector<int> shape;
  int fmt = TF_C64;   // storage format of the tensor
};
// bytes of one tensor element in a storage format (TF_F32: complex FP32)
inline double elem_bytes(int fmt) { return fmt == TF_F32 ? 8.0 : 16.0; }

long long prod_range(const std::vector<int>& s, int a, int b) {
  long long r = 1;
  for (int i = a; i < b; ++i) r *= s[i];
  return r;
}

struct ProdBatch {
  std::vector<ProdDesc> h;
  ProdDesc* d = nullptr;
  long long nblocks = 0;
  int maxn = 0;
  int prec = 0;                  // 0 FP64, 1 split FP32, 2 split FP32 compensated
  double flops = 0, bytes = 0;   // algorithmic work of one launch
  void add(const cplx* X, cplx* Y, const cplx* M, int ldm, int conjT, const std::vector<int>& shape, int mode,
           int nout, cplx alpha, int accumulate, int xfmt = TF_C64, int yfmt = TF_C64) {
    if (yfmt != TF_C64 && (accumulate || alpha.x != 1.0 || alpha.y != 0.0))
      throw StatusError(MCTDH_EARG, "split-format output needs alpha = 1 without accumulation");
    ProdDesc pd;
    memset(&pd, 0, sizeof(pd));
    pd.xfmt = xfmt;
    pd.yfmt = yfmt;
    pd.X = X;
    pd.Y = Y;
    pd.M = M;
    pd.ldm = ldm;
    pd.conjT = conjT;
    pd.L = prod_range(shape, 0, mode);
    pd.R = prod_range(shape, mode + 1, (int)shape.size());
    if (pd.L * pd.R >= (1LL << 31))
      throw StatusError(MCTDH_EUNSUPPORTED, "more than 2^31 fibres in one mode product");
    pd.nin = shape[mode];
    pd.nout = nout;
    pd.alpha = alpha;
    pd.accumulate = accumulate;
    h.push_back(pd);
  }
  void finalize(DevArena& ar) {
    nblocks = 0;
    maxn = 0;
    flops = bytes = 0;
    for (auto& pd : h) {
      pd.block_start = nblocks;
      nblocks += (pd.L * pd.R + 127) / 128;
      maxn = std::max(maxn, std::max(pd.nin, pd.nout));
      const double fib = (double)pd.L * (double)pd.R;
      flops += 8.0 * pd.nin * pd.nout * fib;
      bytes += (elem_bytes(pd.xfmt) * pd.nin + elem_bytes(pd.yfmt) * pd.nout * (pd.accumulate ? 2 : 1)) * fib;
    }
    d = upload_vec(ar, h);
  }
};

// Blocks per contraction: one block per HOLE_TPB fibre tiles, at most HOLE_CAP
// blocks; the partial buffers hold up to HOLE_NBLK_MAX blocks so that the
// ensemble autotuner can re-tile without re-planning.
#define HOLE_TPB 8
#define HOLE_CAP 64
#define HOLE_NBLK_MAX 128
inline int hole_nblk(long long ntiles, int tpb, int cap) {
  return (int)std::min<long long>(std::max<long long>(ntiles / tpb, 1), std::min(cap, HOLE_NBLK_MAX));
}

struct HoleBatch {
  std::vector<HoleDesc> h;
  HoleDesc* d = nullptr;
  long long nblocks = 0;
  int prec = 0;                  // 0 FP64, 2 compensated split FP32
  double flops = 0, bytes = 0;
  // returns index of the hole
  int add(DevArena& ar, const cplx* X, const cplx* Y, long long L, long long R, int n1, int n2,
          int xfmt = TF_C64, int yfmt = TF_C64) {
    HoleDesc hd;
    memset(&hd, 0, sizeof(hd));
    hd.X = X;
    hd.Y = Y;
    hd.xfmt = xfmt;
    hd.yfmt = yfmt;
    hd.L = L;
    hd.R = R;
    if (L * R >= (1LL << 31)) throw StatusError(MCTDH_EUNSUPPORTED, "more than 2^31 fibres in one contraction");
    hd.n1 = n1;
    hd.n2 = n2;
    long long ntiles = (L * R + HOLE_TILE - 1) / HOLE_TILE;
    hd.nblk = hole_nblk(ntiles, HOLE_TPB, HOLE_CAP);
    hd.partial = ar.calloc_c((long long)hole_nblk(ntiles, 1, HOLE_NBLK_MAX) * n1 * n2);
    h.push_back(hd);
    return (int)h.size() - 1;
  }
  void finalize(DevArena& ar) {
    nblocks = 0;
    flops = bytes = 0;
    for (auto& hd : h) {
      hd.block_start = nblocks;
      nblocks += hd.nblk;
      const double fib = (double)hd.L * (double)hd.R;
      flops += 8.0 * hd.n1 * hd.n2 * fib;
      bytes += (elem_bytes(hd.xfmt) * hd.n1 + (hd.X == hd.Y ? 0.0 : elem_bytes(hd.yfmt) * hd.n2)) * fib;
    }
    d = upload_vec(ar, h);
  }
  // new block counts (one block per `tpb` tiles, at most `cap`), in place on the device
  void retile(int tpb, int cap, cudaStream_t st) {
    if (h.empty()) return;
    nblocks = 0;
    for (auto& hd : h) {
      hd.nblk = hole_nblk((hd.L * hd.R + HOLE_TILE - 1) / HOLE_TILE, tpb, cap);
      hd.block_start = nblocks;
      nblocks += hd.nblk;
    }
    CK(cudaMemcpyAsync(d, h.data(), sizeof(HoleDesc) * h.size(), cudaMemcpyHostToDevice, st));
  }
};

struct RedBatch {
  std::vector<RedTarget> tg;
  std::vector<RedTerm> terms;
  std::vector<std::vector<RedTerm>> pending;
  RedTarget* d_tg = nullptr;
  RedTerm* d_terms = nullptr;
  int add_target(cplx* out, int n1, int n2, int ld, int hermitize, int accumulate = 0) {
    RedTarget t;
    memset(&t, 0, sizeof(t));
    t.out = out;
    t.n1 = n1;
    t.n2 = n2;
    t.ld = ld;
    t.hermitize = hermitize;
    t.accumulate = accumulate;
    tg.push_back(t);
    pending.emplace_back();
    return (int)tg.size() - 1;
  }
  void add_term(int target, const HoleDesc& hd, cplx alpha, int conjT = 0) {
    RedTerm rt;
    memset(&rt, 0, sizeof(rt));
    rt.partial = hd.partial;
    rt.nblk = hd.nblk;
    rt.alpha = alpha;
    rt.conjT = conjT;
    pending[target].push_back(rt);
  }
  void finalize(DevArena& ar) {
    terms.clear();
    for (size_t i = 0; i < tg.size(); ++i) {
      tg[i].first = (int)terms.size();
      tg[i].count = (int)pending[i].size();
      for (auto& r : pending[i]) terms.push_back(r);
    }
    d_tg = upload_vec(ar, tg);
    d_terms = upload_vec(ar, terms);
  }
  // block counts of the terms whose partials belong to re-tiled contractions
  void sync_nblk(const std::vector<const HoleBatch*>& hbs, cudaStream_t st) {
    if (terms.empty()) return;
    bool changed = false;
    for (auto& rt : terms)
      for (const HoleBatch* hb : hbs)
        for (const auto& hd : hb->h)
          if (hd.partial == rt.partial && rt.nblk != hd.nblk) {
            rt.nblk = hd.nblk;
            changed = true;
          }
    if (changed) CK(cudaMemcpyAsync(d_terms, terms.data(), sizeof(RedTerm) * terms.size(), cudaMemcpyHostToDevice, st));
  }
};

// Holes whose partials must be finalised before the reduce: the hole descriptors
// are finalised first, then the reduce terms are built from them.
struct HoleRef {
  int hole;
  int target;
  cplx alpha;
  int conjT = 0;   // add the hole's matrix conjugate-transposed
};

// Plan of one overlap evaluation <Psi1|Psi2> / norms (norm_wf, WF_Ovl, DeltaPsi).
struct OvlPlan {
  HoleBatch spf_holes;           // SPF overlap matrices
  RedBatch spf_red;
  std::vector<GwpOvlDesc> gwp_h; // Gaussian-mode overlap matrices
  GwpOvlDesc* gwp_d = nullptr;
  std::vector<ProdBatch> chain;  // one batch per mode step
  HoleBatch dots;
  RedBatch dot_red;
  cplx* d_result = nullptr;      // [3 npk] o11, o22, o12 per packet
  int npk = 1;
};

struct DotPlan {
  cplx* res = nullptr;
  cplx* partial = nullptr;     // DOT_BLOCKS block sums
  unsigned* counter = nullptr; // blocks done (reset by the last one)
};

enum { KP_PROD, KP_HOLE, KP_RED, KP_H1, KP_REGINV, KP_TERMSUM, KP_SPF, KP_ELEM, KP_GWP, KP_N };
struct KProf {
  double ms = 0, flops = 0, bytes = 0;
  long long launches = 0;
};
struct PendingEv {
  int kid;
  cudaEvent_t a, b;
  double flops, bytes;
};

struct Ctx {
  bool ops_fresh = false;    // operators/mean fields at d_y are in place (time ops_fresh_t)
  double ops_fresh_t = -1.0;
  bool profiling = false;
  // the reference's eight named routine timers (timingmod.f90:20-27) on CUDA
  // events: accumulated device time and calls per routine
  bool timing = false;
  double rt_ms[8] = {};
  long long rt_calls[8] = {};
  struct RtEv { int id; cudaEvent_t a, b; bool call; };
  std::vector<RtEv> rt_pending;
  // CUDA graphs of launch sequences that repeat with the same buffers: (kind, key
  // buffer) -> (executable graph, kernel launches it holds)
  struct GraphRec {
    cudaGraphExec_t exec;
    long long launches, eoms, hbs;   // what one replay accounts for
  };
  std::map<std::pair<int, const void*>, GraphRec> graphs;
  std::set<std::pair<int, const void*>> graph_seen;   // run once directly before capture
  bool graphs_off = false;
  KProf prof[KP_N];
  std::vector<PendingEv> pending;
  std::vector<cudaEvent_t> evpool;
  cudaEvent_t user_ev[16] = {};
  std::map<std::pair<const void*, const void*>, DotPlan*> dots;
  bool fsal_valid = false;   // Dormand-Prince derivative carried between steps
  // Adams PECE (integrator.f90:227-380)
  int int_order = 4, int_par1 = 0;
  bool ad_planned = false, ad_valid = false;
  int ad_iprop = 0;                  // bootstrap steps done (propagator.f90:156-181)
  std::vector<cplx*> ad_hist;        // dA_prev(:, 1..order): derivatives at x_(n-1), x_(n-2), ...
  std::vector<double> ad_hprev;      // h_prev(1..order)
  cplx *ad_dcur = nullptr, *ad_temp = nullptr, *ad_new = nullptr, *ad_new1 = nullptr, *ad_dnew = nullptr,
       *ad_d1 = nullptr;
  OvlPlan ad_plan;                   // DeltaPsi(ANew, ANew1)
  // Bulirsch-Stoer (integrator.f90:384-608)
  bool bs_planned = false, bs_first = true;
  int bs_kmax = 0, bs_kopt = 0;
  double bs_tnew = -1e16, bs_hnext = -1e15;
  double bs_Ak[10] = {}, bs_tstore[10] = {};
  double bs_alf[9][9] = {};
  cplx *bs_save = nullptr, *bs_d0 = nullptr, *bs_am = nullptr, *bs_an = nullptr, *bs_sw = nullptr, *bs_d = nullptr,
       *bs_seq = nullptr, *bs_a0 = nullptr, *bs_a1 = nullptr;
  cplx* bs_q[10] = {};
  OvlPlan bs_plan;                   // DeltaPsi(A0, A1) of the extrapolation
  // model
  int nstates = 0, nmodes = 0, ndof = 0, nham = 0, maxdof = 0, nopermax = 0;
  std::vector<int> nspf;  // [m + nmodes*s]
  std::vector<int> nmodedof, multiset, is_gwp, ngp;
  std::vector<std::vector<int>> mode_dofs;
  std::vector<cplx> ae;
  std::vector<int> lhs, rhs, noper, ioper, is_identity, skip_term;
  std::vector<std::vector<std::vector<int>>> oper;  // [m][k] -> {l, r, codes...}
  std::vector<long long> naconf, aoff, ipsi;
  long long naconftot = 0, dimpsi = 0, ntot = 0;
  // statistical mixture: npk packets stored packet-minor per state (state s holds
  // naconf[s] = npk * n1[s] coefficients, packet W at aoff[s] + W * n1[s]); the
  // host arrays are packet-major (APacketOffset(W) = W * nAConftot, aoff1)
  int npk = 1;
  double eps_pop = 1e-6;
  std::vector<long long> n1, aoff1;
  long long n1tot = 0;
  // term kinds: 0 Hamiltonian, 1 type-1 dissipative (operator diss1_of[t]), 2 type-2
  std::vector<int> kind, diss1_of;
  int ndiss1 = 0, ndiss2_terms = 0;
  std::vector<double> aeD1;
  bool mixture = false;       // several packets or dissipation: derivative-based integrators only
  bool skip_mult = false;     // observables: the EOM without the Lagrange multipliers
  // packet stage (plan_packets)
  struct SumPlan {
    SumRange* ranges = nullptr;
    SumSrc* srcs = nullptr;
    int n = 0, nsrc = 0;
  };
  SumPlan pk_sum2;                      // X A (type-2 terms)
  std::vector<SumPlan> pk_sum1;         // V_k A per type-1 operator
  cplx *pk_xa = nullptr, *pk_va = nullptr, *pk_aux = nullptr, *pk_vmix = nullptr;
  PkState* pk_st = nullptr;
  PkGramPair* pk_pairs = nullptr;
  bool pk_on = false;
  int pk_npairs = 0, pk_nmix = 0;
  cplx* pk_partial = nullptr;
  cplx* pk_coef_buf = nullptr;
  PkCoefArgs pk_args;
  PkMix* pk_mix = nullptr;
  std::vector<PkMix> pk_mult_h;
  PkMix* pk_mult = nullptr;
  cplx* pk_mult_out = nullptr;          // output the uploaded multiplier descriptor points at
  std::vector<ProdBatch> aux_chains;    // right chains on AuxA_k (type-1 mean fields)
  HoleBatch aux_holes;
  RedBatch aux_red;
  std::vector<int> modes_dvr;
  std::vector<int> gmode;  // grid size G of DVR modes
  double eps_rho = 1e-8, eps_ovl = 1e-8, eps_C = 1e-8, eps_int = 1e-8, eps_A = 1e-8, eps_psi = 1e-8;
  double min_stepsize = 0, writetime = 0;
  cplx der = mkc(0, -1);
  int int_type_psi = 1;
  int precision = 0;
  int hole_prec = 0;   // single-hole contractions: 0 FP64, 1 FP32 sums, 2 compensated FP32
  int mf_hole_prec = 0;   // the mean-field ones (densities keep hole_prec)
  int hb_prec = 0;     // H_B * B products of the Lanczos steps: 0 FP64, 1 FP32, 2 compensated FP32
  bool reginv_cold = false;   // regularised inverses without the Jacobi warm start
  std::string last_error;
  long long launches = 0;
  long long eom_count = 0, hb_count = 0;

  cudaStream_t st = nullptr;
  bool own_stream = true;   // false for ensemble members (the ensemble's stream)
  // a second stream for CMF2 work that runs beside the Lanczos build (own contexts only)
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool member = false;      // ensemble member: RK only, state vectors owned by the ensemble
  DevArena ar;
  int* d_status = nullptr;
  cplx* d_y = nullptr;      // resident state [A | psi]
  cplx* d_y0 = nullptr;     // start state (for C(t))
  cplx* d_in = nullptr;     // EOM input
  cplx* d_out = nullptr;    // EOM output scratch
  cplx* d_k[7] = {};
  cplx* d_tmp = nullptr;
  cplx* d_err = nullptr;
  cplx* d_hb = nullptr;     // H*B output
  double* d_scal = nullptr; // small scalars: [0] the RK step of the current attempt
  double* h_scal = nullptr; // pinned host staging for d_scal
  long long* d_off1 = nullptr;   // {0, ntot}: the whole vector as one segment

  // DVR operator matrices on device: (dof, code) -> pointer
  std::map<std::pair<int, int>, cplx*> dofmat;
  std::map<std::pair<int, int>, float2*> dofmatf;   // real coefficients split into FP32 (hi, lo)
  std::map<std::pair<int, int>, int> dofkind;

  // per (mode, op) storage
  std::vector<std::vector<cplx*>> hmat, ophi, mf, rhom1mf;  // [m][k]
  std::vector<std::vector<cplx*>> rho;                      // [m][s]
  std::vector<cplx*> rho_ave;                               // [m]

  // EOM plan
  std::vector<H1Desc> h1_h;
  H1Desc* h1_d = nullptr;
  size_t h1_smem = 0;
  int h1_maxn2 = 0;
  std::vector<ProdBatch> chains;  // per depth
  std::vector<ProdBatch> chains_full;   // per depth: right chains needed only for dA (adjoint partners)
  HoleBatch holes;       // mean-field contractions of the general terms
  HoleBatch rho_holes;   // density matrices (FP64 always)
  RedBatch red;
  std::vector<RegInvDesc> reg_h;
  std::vector<MFOp> mfop_h;
  RegInvDesc* reg_d = nullptr;
  MFOp* mfop_d = nullptr;
  std::vector<SpfDesc> spf_h;
  std::vector<SpfOp> spfop_h;
  SpfDesc* spf_d = nullptr;
  SpfOp* spfop_d = nullptr;
  size_t spf_smem = 0;
  long long spf_tiles = 0;
  int spf_nf = 0;          // largest SPF count of the SPF derivative blocks and their operators
  std::vector<SumRange> sum_h;
  std::vector<SumSrc> src_h;
  SumRange* sum_d = nullptr;
  SumSrc* src_d = nullptr;
  // pre-summed same-state single-mode operators
  std::vector<int> term_single;      // mode of a same-state single-mode term, -1 none, -2 general
  std::vector<int> general_terms;
  std::vector<cplx> c0;              // sum of the pure-electronic same-state coefficients per state
  std::vector<MatSumDesc> msum_h;
  std::vector<MatSumSrc> msum_src_h;
  MatSumDesc* msum_d = nullptr;
  MatSumSrc* msum_src_d = nullptr;
  std::map<std::pair<int, int>, cplx*> gmat;   // (s, m) -> G_{s,m}
  ProdBatch gprods;                            // G_{s,m} x_m A_s
  // H_B * B plan for CMF2 (Calc_DHD_B): reads d_hbin, writes d_hb
  cplx* d_hbin = nullptr;
  cplx* d_hbin32 = nullptr;   // precision 1: d_hbin as complex FP32, the input of the H_B products
  cplx* d_in32 = nullptr;     // precision 1: the coefficients of d_in as complex FP32 (chain inputs)
  // compensated contractions (and precision-2 chains): the coefficients of d_in as
  // FP32 split pairs, converted once per evaluation instead of at every staging
  cplx* d_insplit = nullptr;
  FusedDot hb_dot{nullptr, nullptr, nullptr, nullptr};    // <d_hbin | H_B d_hbin> in the term sum
  FusedDot lan_nrm{nullptr, nullptr, nullptr, nullptr};   // ||Kn||^2 in the Lanczos axpy
  std::vector<ProdBatch> hb_chains;
  std::vector<SumSrc> hbsrc_h;
  SumSrc* hbsrc_d = nullptr;
  SumRange* hbsum_d = nullptr;
  // ophi-only h1 plan (CMF2 SPF sweeps: operators on the current SPFs, mean fields frozen)
  std::vector<std::vector<int>> h1_of_mode;  // indices into h1_h per DVR mode
  // overlap plans
  OvlPlan dpsi_plan;   // d_tmp vs d_err
  OvlPlan cmf_ovl;     // CMF2's SPF error: d_ovl1 vs d_ovl2 (own buffers: it runs beside the SPF sweep)
  cplx* d_ovl1 = nullptr;
  std::map<std::tuple<int, int, int>, cplx*> ovl_pool;   // shared overlap-chain buffers (state, chain, parity)
  cplx* d_ovl2 = nullptr;
  OvlPlan pk_norm;     // packet norms of d_in (mixtures with dissipation)
  OvlPlan auto_plan;   // d_y0 vs d_y (o12), d_y norm (o22)
  OvlPlan io_plan;     // d_in vs d_out (host API norm/ovl)
  // CMF2 / Lanczos
  cplx* d_krylov = nullptr;  // [ntotA x 21]
  double* d_lan = nullptr;   // alpha[20], beta[20], evals[20], evecs[400]
  int lan_nk = 0;
  std::vector<double> lan_evals, lan_evecs;
  cplx* d_coef = nullptr;

  // Gaussian (G-MCTDH) modes
  std::vector<int> modes_gwp;
  std::vector<int> gwp_of;                            // mode -> index among Gaussian modes (-1: grid)
  double* gwpa_d = nullptr;                           // GWPa(lda, ns00max, nmodgwp)
  int gwp_lda = 0, ns00max = 0;
  std::vector<std::vector<std::vector<cplx*>>> s00;   // [i][s1][s2] overlap matrices
  std::vector<std::vector<cplx*>> s00m1;              // [i][s] Tikhonov inverses
  std::vector<GwpOvlDesc> gs_h;
  GwpOvlDesc* gs_d = nullptr;
  std::vector<RegInvDesc> gsreg_h;
  RegInvDesc* gsreg_d = nullptr;
  std::vector<GwpH1Desc> gh1_h;
  GwpH1Desc* gh1_d = nullptr;
  std::vector<ProdBatch> gwp_rho_chain;               // S-weighted A for the density matrices
  std::vector<GwpCYDesc> cy_h;
  GwpCYDesc* cy_d = nullptr;
  std::vector<GwpYOp> yop_h;
  GwpYOp* yop_d = nullptr;
  int cy_maxG = 0, cy_maxn = 0, cy_maxops = 0;
  cplx* cy_part = nullptr;                            // per-operator partial sums of Y
  std::vector<std::vector<cplx*>> tau;                // [i][s]
  std::vector<std::vector<cplx*>> dhd;                // [i][k] D^H h D of the CMF2 Lanczos (Calc_DHD)
  // expectation operators (Expectation, output.f90:449-500)
  int nexpect = 0;
  std::vector<int> exp_nterms, exp_lhs, exp_rhs, exp_ioper;   // exp_ioper[m + nmodes * term]
  std::vector<cplx> exp_ae;
  std::vector<std::vector<char>> ham_op;              // [m][k]: the operator of some Hamiltonian term
  std::vector<H1Desc> xh1_h;                          // grid-mode operators of expectation operators only
  H1Desc* xh1_d = nullptr;
  std::vector<GwpH1Desc> xgh1_h;                      // Gaussian-mode ones
  GwpH1Desc* xgh1_d = nullptr;
  cplx* d_adot = nullptr;                             // f * sum_t ae_t H_t A before the corrections
  cplx* d_dA = nullptr;                               // dA after S^-1 and tau
  std::vector<ProdBatch> gwp_sinv;                    // S^-1 products, one batch per Gaussian mode
  std::vector<ProdBatch> gwp_tau;                     // -tau x_m A, one batch per Gaussian mode

  ~Ctx() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second.exec);
    if (h_scal) cudaFreeHost(h_scal);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (st2) cudaStreamDestroy(st2);
  }
  int m_of(int m, int s) const { return nspf[m + nmodes * s]; }
  // tensor shape of state s; a mixture adds the packet index as the slowest dimension
  std::vector<int> shape_of(int s) const {
    std::vector<int> v(nmodes);
    for (int m = 0; m < nmodes; ++m) v[m] = m_of(m, s);
    if (npk > 1) v.push_back(npk);
    return v;
  }
  void count(int n = 1) { launches += n; }
};

// ---------------------------------------------------------------------------
// Set-up
// ---------------------------------------------------------------------------
void load_setup(Ctx& c, const mctdh_setup_t* s) {
  c.nstates = (int)s->nstates;
  c.nmodes = (int)s->nmodes;
  c.ndof = (int)s->ndof;
  c.nham = (int)s->nham;
  c.maxdof = (int)s->maxdof;
  c.nopermax = (int)s->nopermax;
  if (c.nstates < 1 || c.nmodes < 1 || c.nham < 1) throw StatusError(MCTDH_EARG, "empty model");
  c.nspf.resize(c.nmodes * c.nstates);
  for (int i = 0; i < c.nmodes * c.nstates; ++i) c.nspf[i] = (int)s->nspf[i];
  c.nmodedof.resize(c.nmodes);
  c.multiset.resize(c.nmodes);
  c.is_gwp.resize(c.nmodes);
  c.mode_dofs.resize(c.nmodes);
  for (int m = 0; m < c.nmodes; ++m) {
    c.nmodedof[m] = (int)s->nmodedof[m];
    c.multiset[m] = (int)s->multiset[m];
    c.is_gwp[m] = (int)s->is_gwp[m];
    for (int k = 0; k < c.nmodedof[m]; ++k) c.mode_dofs[m].push_back((int)s->idof[k + c.maxdof * m]);
    if (c.is_gwp[m] && c.nmodedof[m] > GWP_MAXDOF)
      throw StatusError(MCTDH_EUNSUPPORTED, "too many DOFs in one Gaussian mode");
    if (!c.is_gwp[m] && c.nmodedof[m] > MAXDOF_MODE) throw StatusError(MCTDH_EUNSUPPORTED, "too many DOFs in one DVR mode");
    for (int st = 0; st < c.nstates; ++st)
      if (c.m_of(m, st) > MAXN_SPF || c.m_of(m, st) < 1)
        throw StatusError(MCTDH_EUNSUPPORTED, "SPF count outside 1..32");
  }
  c.ngp.resize(c.ndof);
  for (int d = 0; d < c.ndof; ++d) c.ngp[d] = (int)s->ngp[d];
  c.ae.resize(c.nham);
  c.lhs.resize(c.nham);
  c.rhs.resize(c.nham);
  for (int t = 0; t < c.nham; ++t) {
    c.ae[t] = mkc(s->ae[2 * t], s->ae[2 * t + 1]);
    c.lhs[t] = (int)s->lhs_el[t];
    c.rhs[t] = (int)s->rhs_el[t];
  }
  c.noper.resize(c.nmodes);
  c.oper.resize(c.nmodes);
  const int w = 2 + c.maxdof;
  for (int m = 0; m < c.nmodes; ++m) {
    c.noper[m] = (int)s->noper[m];
    for (int k = 0; k < c.noper[m]; ++k) {
      std::vector<int> v;
      for (int q = 0; q < 2 + c.nmodedof[m]; ++q) v.push_back((int)s->oper[q + w * (k + c.nopermax * m)]);
      c.oper[m].push_back(v);
    }
  }
  c.ioper.resize(c.nmodes * c.nham);
  c.skip_term.resize(c.nmodes * c.nham);
  for (int i = 0; i < c.nmodes * c.nham; ++i) {
    c.ioper[i] = (int)s->ioper[i];
    c.skip_term[i] = (int)s->skip_term[i];
  }
  c.is_identity.resize(c.nmodes * c.nopermax);
  for (int i = 0; i < c.nmodes * c.nopermax; ++i) c.is_identity[i] = (int)s->is_identity[i];
  // Operators no Hamiltonian term uses (those of expectation operators only) get no
  // mean field and stay out of the EOM; the reference carries them with zero mean
  // fields, which add exact zeros to its sums.
  c.ham_op.assign(c.nmodes, std::vector<char>(c.nopermax, 0));
  for (int t = 0; t < c.nham; ++t)
    for (int m = 0; m < c.nmodes; ++m) {
      const int k = c.ioper[m + c.nmodes * t];
      if (k < 0 || k >= c.noper[m]) throw StatusError(MCTDH_EARG, "iOper out of range");
      c.ham_op[m][k] = 1;
    }
  c.nexpect = (int)s->nexpect;
  if (c.nexpect < 0) throw StatusError(MCTDH_EARG, "nexpect < 0");
  if (c.nexpect > 0) {
    if (!s->expect_nterms || !s->expect_ae || !s->expect_lhs || !s->expect_rhs || !s->expect_ioper)
      throw StatusError(MCTDH_EARG, "expectation operators need their term arrays");
    int tot = 0;
    for (int i = 0; i < c.nexpect; ++i) {
      c.exp_nterms.push_back((int)s->expect_nterms[i]);
      if (c.exp_nterms.back() < 0) throw StatusError(MCTDH_EARG, "negative term count");
      tot += c.exp_nterms.back();
    }
    for (int g = 0; g < tot; ++g) {
      c.exp_ae.push_back(mkc(s->expect_ae[2 * g], s->expect_ae[2 * g + 1]));
      c.exp_lhs.push_back((int)s->expect_lhs[g]);
      c.exp_rhs.push_back((int)s->expect_rhs[g]);
      if (c.exp_lhs.back() < 0 || c.exp_lhs.back() >= c.nstates || c.exp_rhs.back() < 0 ||
          c.exp_rhs.back() >= c.nstates)
        throw StatusError(MCTDH_EARG, "electronic label of an expectation term out of range");
      for (int m = 0; m < c.nmodes; ++m) {
        const int k = (int)s->expect_ioper[m + (long long)c.nmodes * g];
        if (k < 0 || k >= c.noper[m]) throw StatusError(MCTDH_EARG, "iOperExtra out of range");
        c.exp_ioper.push_back(k);
      }
    }
  }
  // statistical mixtures and dissipation (input.f90:156, 216-229, 262, 596-616)
  c.npk = s->npackets > 1 ? (int)s->npackets : 1;
  if (c.npk > MAX_PACKETS) throw StatusError(MCTDH_EUNSUPPORTED, "more than 16 wave packets");
  c.eps_pop = s->eps_pop > 0.0 ? s->eps_pop : 1e-6;
  c.kind.assign(c.nham, 0);
  c.diss1_of.assign(c.nham, -1);
  c.ndiss1 = s->term_kind ? (int)s->ndiss1 : 0;
  if (c.ndiss1 < 0 || c.ndiss1 > MAX_DISS1) throw StatusError(MCTDH_EUNSUPPORTED, "0..4 type-1 dissipative operators");
  if (c.ndiss1 > 0 && !s->diss1_ae) throw StatusError(MCTDH_EARG, "type-1 operators need diss1_ae");
  for (int k = 0; k < c.ndiss1; ++k) c.aeD1.push_back(s->diss1_ae[k]);
  if (s->term_kind) {
    for (int t = 0; t < c.nham; ++t) {
      const int kd = (int)s->term_kind[t];
      if (kd < 0 || kd > 2) throw StatusError(MCTDH_EARG, "term_kind outside 0..2");
      c.kind[t] = kd;
      if (kd == 2) ++c.ndiss2_terms;
      if (kd == 1) {
        const int k = s->term_diss1 ? (int)s->term_diss1[t] : -1;
        if (k < 0 || k >= c.ndiss1) throw StatusError(MCTDH_EARG, "term_diss1 out of range");
        if (c.lhs[t] != c.rhs[t])
          for (int m = 0; m < c.nmodes; ++m)
            if (c.m_of(m, c.lhs[t]) != c.m_of(m, c.rhs[t]))
              throw StatusError(MCTDH_EUNSUPPORTED, "type-1 terms between states need equal SPF counts");
        c.diss1_of[t] = k;
      }
    }
  }
  c.mixture = c.npk > 1 || c.ndiss1 > 0 || c.ndiss2_terms > 0;
  c.naconf.resize(c.nstates);
  c.aoff.resize(c.nstates);
  c.n1.resize(c.nstates);
  c.aoff1.resize(c.nstates);
  long long off = 0;
  for (int st = 0; st < c.nstates; ++st) {
    long long n = 1;
    for (int m = 0; m < c.nmodes; ++m) n *= c.m_of(m, st);
    c.n1[st] = n;
    c.aoff1[st] = c.n1tot;
    c.n1tot += n;
    c.naconf[st] = n * c.npk;
    c.aoff[st] = off;
    off += n * c.npk;
  }
  c.naconftot = off;
  c.dimpsi = s->dimpsi;
  c.ntot = c.naconftot + c.dimpsi;
  c.ipsi.resize(c.nmodes * c.nstates);
  for (int i = 0; i < c.nmodes * c.nstates; ++i) c.ipsi[i] = s->ipsispf[i];
  c.gmode.assign(c.nmodes, 0);
  c.gwp_of.assign(c.nmodes, -1);
  for (int m = 0; m < c.nmodes; ++m) {
    if (c.is_gwp[m]) {
      c.gwp_of[m] = (int)c.modes_gwp.size();
      c.modes_gwp.push_back(m);
      continue;
    }
    c.modes_dvr.push_back(m);
    int G = 1;
    for (int d : c.mode_dofs[m]) G *= c.ngp[d];
    c.gmode[m] = G;
  }
  c.eps_rho = s->eps_rho;
  c.eps_ovl = s->eps_ovl;
  c.eps_C = s->eps_C;
  c.eps_int = s->eps_int;
  c.eps_A = s->eps_A;
  c.eps_psi = s->eps_psi;
  c.min_stepsize = s->min_stepsize;
  c.writetime = s->writetime;
  c.der = mkc(s->der_factor_re, s->der_factor_im);
  c.int_type_psi = (int)s->int_type_psi;
  c.int_order = (int)s->int_order;
  c.int_par1 = (int)s->int_par1;
  c.reginv_cold = s->reginv_cold != 0;
  c.precision = (int)s->precision;
  if (c.precision < 0 || c.precision > 6) throw StatusError(MCTDH_EARG, "precision must be 0 .. 6");
  // precision 3: the products of precision 1 with FP32-accumulated contractions;
  // 4: FP32 mean-field and A-derivative products, compensated H_B products;
  // 5: compensated mean-field and A-derivative products, FP32 H_B products;
  // 6: precision 1 with FP32-accumulated mean-field contractions (densities compensated)
  c.hole_prec = c.precision == 3 ? 1 : (c.precision ? 2 : 0);
  c.mf_hole_prec = (c.precision == 6) ? 1 : c.hole_prec;
  c.hb_prec = c.precision == 4 ? 2 : (c.precision == 5 || c.precision == 3 || c.precision == 6 ? 1 : c.precision);
  if (c.precision == 3 || c.precision == 4 || c.precision == 6) c.precision = 1;
  if (c.precision == 5) c.precision = 2;
  if (!c.modes_gwp.empty()) {
    // Gaussian widths GWPa(maxdof, ns00max, nmodgwp) (psidef: GWPa, init_calc.f90:1020-1068)
    c.gwp_lda = c.maxdof;
    c.ns00max = (int)s->ns00max;
    if (!s->gwpa || c.ns00max < 1) throw StatusError(MCTDH_EARG, "Gaussian modes need gwpa and ns00max");
    for (int m : c.modes_gwp)
      for (int st = 0; st < c.nstates; ++st)
        if (c.m_of(m, st) > c.ns00max) throw StatusError(MCTDH_EARG, "Gaussian SPF count above ns00max");
    const size_t na = (size_t)c.gwp_lda * c.ns00max * c.modes_gwp.size();
    c.gwpa_d = (double*)c.ar.alloc(sizeof(double) * na);
    CK(cudaMemcpy(c.gwpa_d, s->gwpa, sizeof(double) * na, cudaMemcpyHostToDevice));
    for (int m : c.modes_gwp)
      for (int k = 0; k < c.noper[m]; ++k)
        for (int q = 0; q < c.nmodedof[m]; ++q) {
          const int code = c.oper[m][k][2 + q];
          if (code < -3 || code > 20)
            throw StatusError(MCTDH_EUNSUPPORTED, "primitive operator code " + std::to_string(code) +
                                                      " has no Gaussian integral");
        }
  }

  // primitive DOF operator matrices (dense ones in the zlacrm-from-the-right form
  // with the +i factor of p and qp, hamilton.f90:455-461; diagonal q^k)
  for (int m : c.modes_dvr) {
    for (int k = 0; k < c.noper[m]; ++k) {
      for (int q = 0; q < c.nmodedof[m]; ++q) {
        int code = c.oper[m][k][2 + q];
        int d = c.mode_dofs[m][q];
        if (code == 0) continue;
        auto key = std::make_pair(d, code);
        if (c.dofmat.count(key)) continue;
        int ng = c.ngp[d];
        const double* mats = s->dvr_mats + s->dvr_mat_off[d];
        const double* grid = s->dvr_grid + s->dvr_grid_off[d];
        std::vector<cplx> v;
        int kind;
        if (code == -1 || code == -2 || code == -3) {
          kind = (code == -2) ? 1 : 3;   // d^2/dq^2 real; p and qp carry the factor i
          const double* src = code == -1 ? mats : (code == -2 ? mats + ng * ng : mats + 2 * ng * ng);
          v.resize(ng * ng);
          for (int i = 0; i < ng * ng; ++i) v[i] = (code == -2) ? mkc(src[i], 0.0) : mkc(0.0, src[i]);
        } else if (code >= 1 && code <= 20) {
          kind = 2;
          v.resize(ng);
          for (int i = 0; i < ng; ++i) v[i] = mkc(code == 1 ? grid[i] : pow(grid[i], (double)code), 0.0);
        } else if (code > 200 || code <= -200) {
          // parametrised operators: the diagonal gridOper(:, j, dof) (MultTensDiag) or
          // the projector v v^T built like MultTensProj's dger (hamilton.f90:632-661)
          const int j = (code > 200 ? code : -code) - 201;
          if (!s->grid_oper || j < 0 || j >= s->nopparam || ng > s->ngpmax)
            throw StatusError(MCTDH_EARG, "parametrised operator " + std::to_string(code) + " has no gridOper values");
          const double* gv = s->grid_oper + (size_t)s->ngpmax * ((size_t)j + (size_t)s->nopparam * d);
          if (code > 200) {
            kind = 2;
            v.resize(ng);
            for (int i = 0; i < ng; ++i) v[i] = mkc(gv[i], 0.0);
          } else {
            kind = 1;
            v.resize((size_t)ng * ng);
            for (int a = 0; a < ng; ++a)
              for (int b = 0; b < ng; ++b) v[a + (size_t)ng * b] = mkc(gv[a] * gv[b], 0.0);
          }
        } else if (code == -4) {
          // sin^-2 of a Legendre DVR (operDVR), applied like the other dense matrices
          if (!s->oper_dvr || !s->oper_dvr_off || s->oper_dvr_off[d] < 0)
            throw StatusError(MCTDH_EARG, "sin^-2 on a dof without an operDVR matrix");
          kind = 1;
          const double* src = s->oper_dvr + s->oper_dvr_off[d];
          v.resize((size_t)ng * ng);
          for (int i = 0; i < ng * ng; ++i) v[i] = mkc(src[i], 0.0);
        } else {
          throw StatusError(MCTDH_EUNSUPPORTED, "primitive operator code " + std::to_string(code) + " not supported");
        }
        c.dofmat[key] = upload_vec(c.ar, v);
        c.dofkind[key] = kind;
        std::vector<float2> vf(v.size());
        for (size_t i = 0; i < v.size(); ++i) {
          const double x = (kind == 3) ? v[i].y : v[i].x;
          const float hi = (float)x;
          vf[i] = make_float2(hi, (float)(x - (double)hi));
        }
        c.dofmatf[key] = upload_vec(c.ar, vf);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Gaussian modes: overlaps S00 and their Tikhonov inverses (Calc_S00,
// gmctdh_objects.f90:323-381; Calc_S00m1, :385-404) and the h1mode matrices of
// their operators (hamilton.f90:494-524), identity operators included (their
// h1mode is S00, and the Hamiltonian chains do not skip them).
// ---------------------------------------------------------------------------
const cplx* psi_block(const Ctx& c, const cplx* y, int m, int s) {
  return y + c.naconftot + c.ipsi[m + c.nmodes * s];
}
int set_of(const Ctx& c, int m, int s) { return c.multiset[m] ? s : 0; }

void plan_gwp_setup(Ctx& c) {
  const int f = c.nmodes;
  const int ng = (int)c.modes_gwp.size();
  c.s00.assign(ng, std::vector<std::vector<cplx*>>(c.nstates, std::vector<cplx*>(c.nstates, nullptr)));
  c.s00m1.assign(ng, std::vector<cplx*>(c.nstates, nullptr));
  for (int i = 0; i < ng; ++i) {
    const int m = c.modes_gwp[i];
    const double* a = c.gwpa_d + (size_t)c.gwp_lda * c.ns00max * i;
    const int nsets = c.multiset[m] ? c.nstates : 1;
    for (int s1 = 0; s1 < nsets; ++s1) {
      for (int s2 = 0; s2 < nsets; ++s2) {
        const int n1 = c.m_of(m, s1), n2 = c.m_of(m, s2);
        c.s00[i][s1][s2] = c.ar.calloc_c((long long)n1 * n2);
        GwpOvlDesc d;
        memset(&d, 0, sizeof(d));
        d.xi1 = psi_block(c, c.d_in, m, s1);
        d.xi2 = psi_block(c, c.d_in, m, s2);
        d.a = a;
        d.out = c.s00[i][s1][s2];
        d.nmd = c.nmodedof[m];
        d.lda = c.gwp_lda;
        d.n1 = n1;
        d.n2 = n2;
        d.kind = (s1 == s2) ? 0 : (s1 < s2 ? 1 : 2);
        c.gs_h.push_back(d);
      }
      RegInvDesc rd;
      memset(&rd, 0, sizeof(rd));
      rd.A = c.s00[i][s1][s1];
      rd.n = c.m_of(m, s1);
      rd.regtype = 1;
      rd.eps = c.eps_ovl;
      c.s00m1[i][s1] = c.ar.calloc_c((long long)rd.n * rd.n);
      rd.inv_out = c.s00m1[i][s1];
      c.gsreg_h.push_back(rd);
    }
    // h1mode of every operator of the mode
    c.hmat[m].assign(c.noper[m], nullptr);
    c.ophi[m].assign(c.noper[m], nullptr);
    c.mf[m].assign(c.noper[m], nullptr);
    c.rhom1mf[m].assign(c.noper[m], nullptr);
    for (int k = 0; k < c.noper[m]; ++k) {
      const int l = c.oper[m][k][0], r = c.oper[m][k][1];
      const int n1 = c.m_of(m, l), n2 = c.m_of(m, r);
      c.hmat[m][k] = c.ar.calloc_c((long long)n1 * n2);
      if (!c.is_identity[m + f * k] && c.ham_op[m][k]) c.mf[m][k] = c.ar.calloc_c((long long)n1 * n2);
      GwpH1Desc hd;
      memset(&hd, 0, sizeof(hd));
      hd.xi1 = psi_block(c, c.d_in, m, l);
      hd.xi2 = psi_block(c, c.d_in, m, r);
      hd.a = a;
      hd.S = c.s00[i][set_of(c, m, l)][set_of(c, m, r)];
      hd.out = c.hmat[m][k];
      hd.nmd = c.nmodedof[m];
      hd.lda = c.gwp_lda;
      hd.n1 = n1;
      hd.n2 = n2;
      hd.same_state = (l == r);
      for (int q = 0; q < c.nmodedof[m]; ++q) hd.ops[q] = c.oper[m][k][2 + q];
      if (c.ham_op[m][k]) c.gh1_h.push_back(hd);
      else c.xgh1_h.push_back(hd);
    }
  }
  c.gs_d = upload_vec(c.ar, c.gs_h);
  c.gsreg_d = upload_vec(c.ar, c.gsreg_h);
  c.gh1_d = upload_vec(c.ar, c.gh1_h);
  c.xgh1_d = upload_vec(c.ar, c.xgh1_h);
}

// S-weighted coefficient tensors for the density matrices (Calc_rho1mode,
// gmctdh_objects.f90:408-477): S00 applied on every Gaussian mode except `skip`,
// in the order of the Gaussian modes.  Returns the tensor (A_s itself when no
// product is needed).
const cplx* plan_s_weighted(Ctx& c, int s, int skip) {
  const cplx* cur = c.d_in + c.aoff[s];
  std::vector<int> sh = c.shape_of(s);
  int depth = 0;
  for (int i = 0; i < (int)c.modes_gwp.size(); ++i) {
    const int m = c.modes_gwp[i];
    if (m == skip) continue;
    if ((int)c.gwp_rho_chain.size() <= depth) c.gwp_rho_chain.emplace_back();
    cplx* out = c.ar.calloc_c(c.naconf[s]);
    const int n = sh[m];
    c.gwp_rho_chain[depth].add(cur, out, c.s00[i][set_of(c, m, s)][set_of(c, m, s)], n, 0, sh, m, n, mkc(1, 0), 0);
    cur = out;
    ++depth;
  }
  return cur;
}

// ---------------------------------------------------------------------------
// Planning of the EOM (Calc_Derivs, derivatives.f90:39-237)
// ---------------------------------------------------------------------------
void plan_gwp_derivs(Ctx& c);

void plan_ovl(Ctx& c, OvlPlan& P, cplx* y1, cplx* y2, int prec, bool norm_only = false, bool shared = true);
void run_ovl(Ctx& c, OvlPlan& P);

// type-1 mean-field contribution: contraction of L_im(A) with the right chain on AuxA
struct AuxRef {
  int hole, im, k;
  cplx ae;
};

// Statistical mixtures and dissipation (gmctdh_objects.f90:606-845, 1128-1137;
// derivatives.f90:70-83, 238-242).  After the mean-field reduction of every EOM:
//   X A = sum_t f i aeD2 ae_t W_t A (type-2 terms)   and   V_k A = sum_t ae_t V_t A,
//   the packet norms, G = <A_i|X A_j> and <A_i|V_k A_j> (pk_gram), the populations,
//   multipliers and mixing matrices (pk_coef), D = sum_k V_k A C1_k and
//   AuxA_k = A C2_k (pk_mix), the right chains on AuxA_k and their contractions with
//   the left chains on A, added to the mean fields.  D and X A join the term sum of
//   dA; the multipliers dA += A (multLagDiag I + i multLag) close the EOM.
void plan_packets(Ctx& c, std::vector<std::vector<SumSrc>>& srcs, std::vector<std::vector<SumSrc>>& srcs2,
                  std::vector<std::vector<std::vector<SumSrc>>>& srcs1,
                  const std::map<std::pair<int, int>, int>& mf_target, const std::vector<AuxRef>& arefs) {
  const int P = c.npk;
  const bool has2 = c.ndiss2_terms > 0;
  std::vector<PkState> st(c.nstates);
  for (int s = 0; s < c.nstates; ++s) st[s] = PkState{c.aoff[s], c.n1[s]};
  c.pk_st = upload_vec(c.ar, st);
  auto sum_plan = [&](std::vector<std::vector<SumSrc>>& v, Ctx::SumPlan& sp) {
    std::vector<SumRange> rr;
    std::vector<SumSrc> ss;
    for (int s = 0; s < c.nstates; ++s) {
      SumRange r;
      r.offset = c.aoff[s];
      r.n = c.naconf[s];
      r.first = (int)ss.size();
      r.count = (int)v[s].size();
      for (auto& x : v[s]) ss.push_back(x);
      rr.push_back(r);
    }
    split_coeffs(ss);
    sp.n = (int)rr.size();
    sp.nsrc = (int)ss.size();
    sp.ranges = upload_vec(c.ar, rr);
    sp.srcs = upload_vec(c.ar, ss);
  };
  std::vector<PkGramPair> pairs;
  // WPpop = norm_wf(A_W, psi) with the SPF overlaps (derivatives.f90:70-76): the
  // intermediate states of an integrator step have non-orthonormal SPFs
  if (P > 1) plan_ovl(c, c.pk_norm, c.d_in, c.d_in, 0, true);
  if (has2) {
    c.pk_xa = c.ar.calloc_c(c.naconftot);
    sum_plan(srcs2, c.pk_sum2);
    for (int j = 0; j < P; ++j)
      for (int i = 0; i < P; ++i) pairs.push_back(PkGramPair{c.d_in, c.pk_xa, i, j});
    for (int s = 0; s < c.nstates; ++s) srcs[s].push_back(SumSrc{c.pk_xa + c.aoff[s], mkc(1, 0)});
  }
  c.pk_sum1.resize(c.ndiss1);
  for (int k = 0; k < c.ndiss1; ++k) {
    sum_plan(srcs1[k], c.pk_sum1[k]);
    for (int j = 0; j < P; ++j)
      for (int i = 0; i < P; ++i) pairs.push_back(PkGramPair{c.d_in, c.pk_va + (long long)k * c.naconftot, i, j});
  }
  c.pk_on = true;
  c.pk_npairs = (int)pairs.size();
  c.pk_pairs = upload_vec(c.ar, pairs);
  c.pk_partial = c.ar.calloc_c((long long)c.pk_npairs * PK_GRAM_BLOCKS);
  c.pk_coef_buf = c.ar.calloc_c((long long)(2 * c.ndiss1 + 1) * P * P + P);
  PkCoefArgs& a = c.pk_args;
  memset(&a, 0, sizeof(a));
  a.P = P;
  a.ndiss1 = c.ndiss1;
  a.has2 = has2;
  a.npairs = c.pk_npairs;
  a.eps_pop = c.eps_pop;
  for (int k = 0; k < c.ndiss1; ++k) a.aeD1[k] = c.aeD1[k];
  a.partial = c.pk_partial;
  a.norms = c.pk_norm.d_result;
  a.C1 = c.pk_coef_buf;
  a.C2 = c.pk_coef_buf + (long long)c.ndiss1 * P * P;
  a.ML = c.pk_coef_buf + (long long)2 * c.ndiss1 * P * P;
  a.pop = reinterpret_cast<double*>(a.ML + P * P);
  std::vector<PkMix> mix;
  if (c.ndiss1 > 0) {
    c.pk_vmix = c.ar.calloc_c(c.naconftot);
    for (int k = 0; k < c.ndiss1; ++k)
      mix.push_back(PkMix{c.pk_va + (long long)k * c.naconftot, a.C1 + (long long)k * P * P, c.pk_vmix, k > 0});
    for (int k = 0; k < c.ndiss1; ++k)
      mix.push_back(PkMix{c.d_in, a.C2 + (long long)k * P * P, c.pk_aux + (long long)k * c.naconftot, 0});
    for (int s = 0; s < c.nstates; ++s) srcs[s].push_back(SumSrc{c.pk_vmix + c.aoff[s], mkc(1, 0)});
  }
  c.pk_nmix = (int)mix.size();
  if (!mix.empty()) c.pk_mix = upload_vec(c.ar, mix);
  // type-1 mean fields: added to the reduction's targets, or written where no other
  // term has a mean field for the operator
  for (auto& b : c.aux_chains) {
    b.prec = c.precision;
    b.finalize(c.ar);
  }
  c.aux_holes.prec = c.mf_hole_prec;
  c.aux_holes.finalize(c.ar);
  std::map<std::pair<int, int>, int> tg;
  for (const AuxRef& r : arefs) {
    const auto key = std::make_pair(r.im, r.k);
    if (!tg.count(key)) {
      const int l = c.oper[r.im][r.k][0], rr = c.oper[r.im][r.k][1];
      const int n1 = c.m_of(r.im, l), n2 = c.m_of(r.im, rr);
      tg[key] = c.aux_red.add_target(c.mf[r.im][r.k], n1, n2, n1, 0, mf_target.count(key) ? 1 : 0);
    }
    c.aux_red.add_term(tg[key], c.aux_holes.h[r.hole], r.ae);
  }
  c.aux_red.finalize(c.ar);
  if (P > 1) {
    std::vector<PkMix> mult{PkMix{c.d_in, a.ML, nullptr, 1}};   // output set at run time
    c.pk_mult_h = mult;
    c.pk_mult = upload_vec(c.ar, mult);
  }
}

void plan_eom(Ctx& c) {
  const int f = c.nmodes;
  if (c.mixture) {
    c.pk_va = c.ndiss1 ? c.ar.calloc_c((long long)c.ndiss1 * c.naconftot) : nullptr;
    c.pk_aux = c.ndiss1 ? c.ar.calloc_c((long long)c.ndiss1 * c.naconftot) : nullptr;
  }
  const int nsm = MAXN_SPF;
  (void)nsm;
  c.hmat.assign(f, {});
  c.ophi.assign(f, {});
  c.mf.assign(f, {});
  c.rhom1mf.assign(f, {});
  c.rho.assign(f, std::vector<cplx*>(c.nstates, nullptr));
  c.rho_ave.assign(f, nullptr);
  c.h1_of_mode.assign(f, {});
  // h1mode / ophi descriptors
  size_t smem = 0;
  for (int m : c.modes_dvr) {
    const int G = c.gmode[m];
    c.hmat[m].assign(c.noper[m], nullptr);
    c.ophi[m].assign(c.noper[m], nullptr);
    c.mf[m].assign(c.noper[m], nullptr);
    c.rhom1mf[m].assign(c.noper[m], nullptr);
    for (int k = 0; k < c.noper[m]; ++k) {
      const int l = c.oper[m][k][0], r = c.oper[m][k][1];
      const int n1 = c.m_of(m, l), n2 = c.m_of(m, r);
      c.hmat[m][k] = c.ar.calloc_c((long long)n1 * n2);
      if (c.is_identity[m + f * k]) {
        std::vector<cplx> I(n1 * n2, mkc(0, 0));
        for (int j = 0; j < std::min(n1, n2); ++j) I[j + n1 * j] = mkc(1, 0);
        CK(cudaMemcpy(c.hmat[m][k], I.data(), sizeof(cplx) * I.size(), cudaMemcpyHostToDevice));
        continue;
      }
      const bool ham = c.ham_op[m][k];
      c.ophi[m][k] = c.ar.calloc_c((long long)G * n2);
      if (ham) {
        c.mf[m][k] = c.ar.calloc_c((long long)n1 * n2);
        c.rhom1mf[m][k] = c.ar.calloc_c((long long)n1 * n2);
      }
      H1Desc hd;
      memset(&hd, 0, sizeof(hd));
      hd.phi_r = c.d_in + c.naconftot + c.ipsi[m + f * r];
      hd.phi_l = c.d_in + c.naconftot + c.ipsi[m + f * l];
      hd.ophi = c.ophi[m][k];
      hd.h = c.hmat[m][k];
      hd.X = c.ar.calloc_c((long long)n1 * n2);
      hd.G = G;
      hd.n1 = n1;
      hd.n2 = n2;
      hd.same_state = (l == r);
      hd.ndof = c.nmodedof[m];
      for (int q = 0; q < hd.ndof; ++q) {
        int d = c.mode_dofs[m][q];
        int code = c.oper[m][k][2 + q];
        hd.ng[q] = c.ngp[d];
        if (code == 0) {
          hd.optype[q] = 0;
        } else {
          auto key = std::make_pair(d, code);
          hd.optype[q] = c.dofkind[key];
          hd.mat[q] = c.dofmat[key];
          hd.matf[q] = c.dofmatf[key];
        }
      }
      if (ham) {
        c.h1_of_mode[m].push_back((int)c.h1_h.size());
        c.h1_h.push_back(hd);
      } else {
        c.xh1_h.push_back(hd);
      }
      smem = std::max(smem, sizeof(cplx) * (size_t)(2 * G));
      c.h1_maxn2 = std::max(c.h1_maxn2, n2);
    }
  }
  c.h1_smem = smem;
  c.h1_d = upload_vec(c.ar, c.h1_h);
  c.xh1_d = upload_vec(c.ar, c.xh1_h);
  if (!c.modes_gwp.empty()) plan_gwp_setup(c);

  if (c.hole_prec == 2 && !c.member && c.modes_gwp.empty() && !c.mixture)
    c.d_insplit = c.ar.calloc_c(c.naconftot);
  // the contractions' operand for A itself: its split copy where there is one
  auto hole_in = [&](const cplx* p, int fmt, int s) -> std::pair<const cplx*, int> {
    if (c.d_insplit && p == c.d_in + c.aoff[s]) return std::make_pair((const cplx*)(c.d_insplit + c.aoff[s]), (int)TF_SPLIT);
    return std::make_pair(p, fmt);
  };
  // density matrices (Calc_rho1mode, gmctdh_objects.f90:408-477)
  std::vector<HoleRef> hrefs;       // mean-field contractions (c.holes)
  std::vector<HoleRef> rrefs;       // density-matrix contractions (c.rho_holes, FP64)
  std::vector<std::vector<int>> rho_hole(f, std::vector<int>(c.nstates, -1));
  std::vector<int> rho_modes = c.modes_dvr;
  rho_modes.insert(rho_modes.end(), c.modes_gwp.begin(), c.modes_gwp.end());
  std::map<std::pair<int, int>, const cplx*> weighted;   // (state, skipped Gaussian mode or -1)
  for (int m : rho_modes) {
    int ave_target = -1;
    if (!c.multiset[m]) {
      int n = c.m_of(m, 0);
      c.rho_ave[m] = c.ar.calloc_c((long long)n * n);
      ave_target = c.red.add_target(c.rho_ave[m], n, n, n, 1);
    }
    for (int s = 0; s < c.nstates; ++s) {
      int n = c.m_of(m, s);
      c.rho[m][s] = c.ar.calloc_c((long long)n * n);
      std::vector<int> sh = c.shape_of(s);
      const cplx* Y = c.d_in + c.aoff[s];
      if (!c.modes_gwp.empty()) {
        const auto key = std::make_pair(s, c.is_gwp[m] ? m : -1);
        if (!weighted.count(key)) weighted[key] = plan_s_weighted(c, s, key.second);
        Y = weighted[key];
      }
      const auto hy = hole_in(Y, TF_C64, s), hx = hole_in(c.d_in + c.aoff[s], TF_C64, s);
      int hidx = c.rho_holes.add(c.ar, hy.first, hx.first, prod_range(sh, 0, m),
                                 prod_range(sh, m + 1, (int)sh.size()), n, n, hy.second, hx.second);
      rho_hole[m][s] = hidx;
      int tg = c.red.add_target(c.rho[m][s], n, n, n, 1);
      rrefs.push_back(HoleRef{hidx, tg, mkc(1, 0)});
      if (ave_target >= 0) rrefs.push_back(HoleRef{hidx, ave_target, mkc(1, 0)});
    }
  }
  // Hamiltonian terms (Calc_MeanField, gmctdh_objects.f90:513-601).
  // A same-state term that touches at most one mode (all other modes are the
  // skipped identity) has AL = A and AR = A around that mode, so its mean field
  // is ae * sum conj(A) A -- the very contraction the density matrix is built
  // from -- and its A-derivative is ae * h x_m A.  Such terms reuse the density
  // contraction for the mean field and are pre-summed per (state, mode) into one
  // operator G_{s,m} = sum_t ae_t h_t applied once.  All other terms run the
  // reference's left/right chains.
  c.chains.assign(f + 1, ProdBatch());
  std::vector<std::vector<SumSrc>> srcs(c.nstates);
  // chain intermediates: complex FP32 in precision 1, FP32 split pairs in precision 2
  const int chain_fmt = c.precision == 1 ? TF_F32 : (c.precision ? TF_SPLIT : TF_C64);
  // precision 1: the products read the coefficients converted once to complex FP32
  // (the contractions keep the FP64 coefficients)
  if (c.precision == 1 && !c.member) c.d_in32 = c.ar.calloc_c((c.naconftot + 1) / 2);
  auto prod_in = [&](const TRef& X, int s) -> std::pair<const cplx*, int> {
    if (c.d_in32 && X.p == c.d_in + c.aoff[s])   // 8-byte elements: offsets count float2
      return std::make_pair(reinterpret_cast<const cplx*>(reinterpret_cast<float2*>(c.d_in32) + c.aoff[s]),
                            (int)TF_F32);
    if (c.precision == 2 && c.d_insplit && X.p == c.d_in + c.aoff[s])
      return std::make_pair((const cplx*)(c.d_insplit + c.aoff[s]), (int)TF_SPLIT);
    return std::make_pair((const cplx*)X.p, X.fmt);
  };
  std::map<std::pair<int, int>, int> mf_target;   // (m,k) -> red target
  auto mf_tg = [&](int im, int k) {
    auto key = std::make_pair(im, k);
    if (!mf_target.count(key)) {
      const int l = c.oper[im][k][0], r = c.oper[im][k][1];
      int n1 = c.m_of(im, l), n2 = c.m_of(im, r);
      mf_target[key] = c.red.add_target(c.mf[im][k], n1, n2, n1, 0);
    }
    return mf_target[key];
  };
  // per term kind: 0 Hamiltonian (dA), 2 type-2 dissipation (its own sum X A, needed
  // alone for the Lagrange multipliers)
  std::vector<cplx> c0k[3] = {std::vector<cplx>(c.nstates, mkc(0, 0)), {}, std::vector<cplx>(c.nstates, mkc(0, 0))};
  std::vector<cplx>& c0 = c0k[0];
  std::map<std::pair<int, int>, std::vector<MatSumSrc>> gsumk[3];  // (s, m) -> sum_t ae_t h_t
  std::vector<std::vector<SumSrc>> srcs2(c.nstates);
  std::vector<std::vector<std::vector<SumSrc>>> srcs1(c.ndiss1, std::vector<std::vector<SumSrc>>(c.nstates));
  auto srcs_of = [&](int t) -> std::vector<std::vector<SumSrc>>& {
    return c.kind[t] == 2 ? srcs2 : (c.kind[t] == 1 ? srcs1[c.diss1_of[t]] : srcs);
  };
  std::vector<AuxRef> arefs;
  c.term_single.assign(c.nham, -2);
  // Hermitian-conjugate partners among the cross-state terms: t2 acts from s2 to s1
  // with the same primitive operators as t1 on every mode and the conjugate
  // coefficient.  Every primitive DOF operator is Hermitian (q^k, i d/dq, d^2/dq^2,
  // i (q d/dq + d/dq q), sin^-2, projectors), so on every mode t2's matrix is the
  // adjoint of t1's and each single-hole mean field of t2 is t1's conjugate-
  // transposed: only t1's contractions are computed, and t2's right chain is
  // needed only for its contribution to dA (c.chains_full).
  c.chains_full.assign(f + 1, ProdBatch());
  std::vector<int> leader_of(c.nham, -1), is_general(c.nham, 0);
  {
    for (int t = 0; t < c.nham; ++t) {
      int nact = 0, mact = -1;
      for (int m = 0; m < f; ++m)
        if (!c.skip_term[m + f * t]) { ++nact; mact = m; }
      is_general[t] = c.kind[t] == 1 || !(c.lhs[t] == c.rhs[t] && nact <= 1 && (mact < 0 || !c.is_gwp[mact]));
    }
    std::vector<char> taken(c.nham, 0);
    for (int t2 = 0; t2 < c.nham; ++t2) {
      if (!is_general[t2] || c.lhs[t2] == c.rhs[t2]) continue;
      for (int t1 = 0; t1 < t2; ++t1) {
        if (!is_general[t1] || taken[t1] || leader_of[t1] >= 0) continue;
        if (c.kind[t1] != c.kind[t2] || c.kind[t1] == 1) continue;
        if (c.lhs[t1] != c.rhs[t2] || c.rhs[t1] != c.lhs[t2]) continue;
        const cplx a1 = c.ae[t1], a2 = c.ae[t2];
        const double da = hypot(a2.x - a1.x, a2.y + a1.y), ma = hypot(a1.x, a1.y);
        if (!(da <= 1e-14 * ma)) continue;
        bool same = true;
        for (int m = 0; m < f && same; ++m) {
          if (c.skip_term[m + f * t1] != c.skip_term[m + f * t2]) { same = false; break; }
          const std::vector<int>& o1 = c.oper[m][c.ioper[m + f * t1]];
          const std::vector<int>& o2 = c.oper[m][c.ioper[m + f * t2]];
          const bool el = c.multiset[m] ? (o2[0] == o1[1] && o2[1] == o1[0]) : (o2[0] == o1[0] && o2[1] == o1[1]);
          same = el && std::equal(o1.begin() + 2, o1.end(), o2.begin() + 2);
        }
        if (!same) continue;
        leader_of[t2] = t1;
        taken[t1] = 1;
        break;
      }
    }
  }
  std::map<std::pair<int, int>, int> term_hole;   // (leader term, mode) -> contraction
  for (int t = 0; t < c.nham; ++t) {
    const int s1 = c.lhs[t], s2 = c.rhs[t];
    int nact = 0, mact = -1;
    for (int m = 0; m < f; ++m)
      if (!c.skip_term[m + f * t]) { ++nact; mact = m; }
    if (c.kind[t] != 1 && s1 == s2 && nact <= 1 && (mact < 0 || !c.is_gwp[mact])) {
      c.term_single[t] = c.kind[t] == 0 ? mact : -2;
      if (mact < 0) {
        c0k[c.kind[t]][s1] = cadd(c0k[c.kind[t]][s1], c.ae[t]);
        continue;
      }
      const int k = c.ioper[mact + f * t];
      gsumk[c.kind[t]][std::make_pair(s1, mact)].push_back(MatSumSrc{c.hmat[mact][k], c.ae[t]});
      if (!c.is_identity[mact + f * k]) rrefs.push_back(HoleRef{rho_hole[mact][s1], mf_tg(mact, k), c.ae[t]});
      continue;
    }
    // general term: right chain always reaches R_f; the left chain stops at the
    // last mode whose mean field is needed (an adjoint partner has neither left
    // chain nor contractions, and its right chain serves dA only)
    const int leader = leader_of[t];
    // type-1 terms: the right chain on A serves V A only (gmctdh_objects.f90:628-649);
    // their mean fields contract the left chain with a right chain on AuxA (below)
    std::vector<ProdBatch>& rchains = (leader >= 0 || c.kind[t] == 1) ? c.chains_full : c.chains;
    int lmax = 0;
    for (int im = 0; im < f; ++im)
      if (!c.is_identity[im + f * c.ioper[im + f * t]]) lmax = im;
    if (leader >= 0 || c.kind[t] == 1) lmax = 0;
    std::vector<TRef> R(f + 1), L(f);
    R[0].p = c.d_in + c.aoff[s2];
    R[0].shape = c.shape_of(s2);
    for (int i = 1; i <= f; ++i) {
      const int jm = f - i;
      if (c.skip_term[jm + f * t]) { R[i] = R[i - 1]; continue; }
      const int k = c.ioper[jm + f * t];
      const int n1 = c.m_of(jm, s1);
      std::vector<int> ns = R[i - 1].shape;
      ns[jm] = n1;
      cplx* out = c.ar.calloc_c(prod_range(ns, 0, (int)ns.size()));
      const auto in = prod_in(R[i - 1], s2);
      rchains[i].add(in.first, out, c.hmat[jm][k], n1, 0, R[i - 1].shape, jm, n1, mkc(1, 0), 0, in.second,
                     chain_fmt);
      R[i].p = out;
      R[i].shape = ns;
      R[i].fmt = chain_fmt;
    }
    L[0].p = c.d_in + c.aoff[s1];
    L[0].shape = c.shape_of(s1);
    for (int i = 1; i <= lmax; ++i) {
      const int im = i - 1;
      if (c.skip_term[im + f * t]) { L[i] = L[i - 1]; continue; }
      const int k = c.ioper[im + f * t];
      const int n1 = c.m_of(im, s1), n2 = c.m_of(im, s2);
      std::vector<int> ns = L[i - 1].shape;
      ns[im] = n2;
      cplx* out = c.ar.calloc_c(prod_range(ns, 0, (int)ns.size()));
      const auto in = prod_in(L[i - 1], s1);
      c.chains[i].add(in.first, out, c.hmat[im][k], n1, 1, L[i - 1].shape, im, n2, mkc(1, 0), 0, in.second,
                      chain_fmt);
      L[i].p = out;
      L[i].shape = ns;
      L[i].fmt = chain_fmt;
    }
    if (c.kind[t] == 1) {
      // V_k A = sum_t ae_t V_t A (no der_factor), and the mean fields of
      // gmctdh_objects.f90:694-744: ae_t <V_t^(not im) A_s2 | AuxA_k,s1> over the packets,
      // an (nSPF(s2) x nSPF(s1)) matrix added into the operator's mean field (equal
      // counts).  The operators of the modes below im act on A_s2 (P chain), those
      // above im act adjoint on AuxA_s1 (Q chain): <h_< h_> A | Y> = <h_< A | h_>^H Y>.
      const int k1 = c.diss1_of[t];
      srcs1[k1][s1].push_back(SumSrc{R[f].p, c.ae[t], R[f].fmt});
      int imin = f, imax = -1;
      for (int im = 0; im < f; ++im)
        if (!c.is_identity[im + f * c.ioper[im + f * t]]) {
          imin = std::min(imin, im);
          imax = im;
        }
      std::vector<TRef> Pc(f), Q(f);
      Pc[0].p = c.d_in + c.aoff[s2];
      Pc[0].shape = c.shape_of(s2);
      for (int i = 1; i <= imax; ++i) {
        const int m = i - 1;
        if (c.skip_term[m + f * t]) { Pc[i] = Pc[i - 1]; continue; }
        const int k = c.ioper[m + f * t];
        const int n1 = c.m_of(m, s1);
        std::vector<int> ns = Pc[i - 1].shape;
        ns[m] = n1;
        cplx* out = c.ar.calloc_c(prod_range(ns, 0, (int)ns.size()));
        const auto in = prod_in(Pc[i - 1], s2);
        c.chains[i].add(in.first, out, c.hmat[m][k], n1, 0, Pc[i - 1].shape, m, n1, mkc(1, 0), 0, in.second,
                        chain_fmt);
        Pc[i].p = out;
        Pc[i].shape = ns;
        Pc[i].fmt = chain_fmt;
      }
      Q[0].p = c.pk_aux + (long long)k1 * c.naconftot + c.aoff[s1];
      Q[0].shape = c.shape_of(s1);
      for (int i = 1; i <= f - 1 - imin; ++i) {
        const int jm = f - i;
        if (c.skip_term[jm + f * t]) { Q[i] = Q[i - 1]; continue; }
        const int k = c.ioper[jm + f * t];
        const int n1 = c.m_of(jm, s1), n2 = c.m_of(jm, s2);
        std::vector<int> ns = Q[i - 1].shape;
        ns[jm] = n2;
        cplx* out = c.ar.calloc_c(prod_range(ns, 0, (int)ns.size()));
        if ((int)c.aux_chains.size() <= i) c.aux_chains.resize(i + 1);
        c.aux_chains[i].add(Q[i - 1].p, out, c.hmat[jm][k], n1, 1, Q[i - 1].shape, jm, n2, mkc(1, 0), 0,
                            Q[i - 1].fmt, chain_fmt);
        Q[i].p = out;
        Q[i].shape = ns;
        Q[i].fmt = chain_fmt;
      }
      for (int im = 0; im < f; ++im) {
        const int k = c.ioper[im + f * t];
        if (c.is_identity[im + f * k]) continue;
        const TRef& X = Pc[im];
        const TRef& Y = Q[f - 1 - im];
        long long Ll = prod_range(X.shape, 0, im), Rr = prod_range(X.shape, im + 1, (int)X.shape.size());
        int hidx = c.aux_holes.add(c.ar, X.p, Y.p, Ll, Rr, X.shape[im], Y.shape[im], X.fmt, Y.fmt);
        arefs.push_back(AuxRef{hidx, im, k, c.ae[t]});
      }
      continue;
    }
    srcs_of(t)[s1].push_back(SumSrc{R[f].p, cmul(c.der, c.ae[t]), R[f].fmt});
    c.general_terms.push_back(t);
    for (int im = 0; im < f; ++im) {
      const int k = c.ioper[im + f * t];
      if (c.is_identity[im + f * k]) continue;
      if (leader >= 0) {
        hrefs.push_back(HoleRef{term_hole.at(std::make_pair(leader, im)), mf_tg(im, k), c.ae[t], 1});
        continue;
      }
      const TRef& X = L[im];
      const TRef& Y = R[f - 1 - im];
      long long Ll = prod_range(X.shape, 0, im), Rr = prod_range(X.shape, im + 1, (int)X.shape.size());
      const auto hx = c.mf_hole_prec == 2 ? hole_in(X.p, X.fmt, s1) : std::make_pair((const cplx*)X.p, X.fmt);
      const auto hy = c.mf_hole_prec == 2 ? hole_in(Y.p, Y.fmt, s2) : std::make_pair((const cplx*)Y.p, Y.fmt);
      int hidx = c.holes.add(c.ar, hx.first, hy.first, Ll, Rr, X.shape[im], Y.shape[im], hx.second, hy.second);
      term_hole[std::make_pair(t, im)] = hidx;
      hrefs.push_back(HoleRef{hidx, mf_tg(im, k), c.ae[t]});
    }
  }
  // pre-summed single-mode operators and their products with A
  for (int kd : {0, 2})
  for (auto& kv : gsumk[kd]) {
    const int s = kv.first.first, m = kv.first.second;
    const int n = c.m_of(m, s);
    MatSumDesc md;
    md.out = c.ar.calloc_c((long long)n * n);
    md.n1 = n;
    md.n2 = n;
    md.first = (int)c.msum_src_h.size();
    md.count = (int)kv.second.size();
    for (auto& x : kv.second) c.msum_src_h.push_back(x);
    c.msum_h.push_back(md);
    if (kd == 0) c.gmat[kv.first] = md.out;   // H_B of CMF2 takes the Hamiltonian's operators only
    std::vector<int> sh = c.shape_of(s);
    cplx* out = c.ar.calloc_c(prod_range(sh, 0, (int)sh.size()));
    const int gfmt = c.precision == 1 ? TF_F32 : chain_fmt;   // FP32 products in precision 1
    TRef root;
    root.p = c.d_in + c.aoff[s];
    const auto in = prod_in(root, s);
    c.gprods.add(in.first, out, md.out, n, 0, sh, m, n, mkc(1, 0), 0, in.second, gfmt);
    (kd == 2 ? srcs2 : srcs)[s].push_back(SumSrc{out, c.der, gfmt});
  }
  for (int s = 0; s < c.nstates; ++s) {
    if (c0[s].x != 0.0 || c0[s].y != 0.0) srcs[s].push_back(SumSrc{c.d_in + c.aoff[s], cmul(c.der, c0[s])});
    const cplx c2 = c0k[2][s];
    if (c2.x != 0.0 || c2.y != 0.0) srcs2[s].push_back(SumSrc{c.d_in + c.aoff[s], cmul(c.der, c2)});
  }
  // without dissipation the multipliers vanish and the packets need no extra stage
  if (c.ndiss1 > 0 || c.ndiss2_terms > 0) plan_packets(c, srcs, srcs2, srcs1, mf_target, arefs);
  c.c0 = c0;
  c.msum_d = upload_vec(c.ar, c.msum_h);
  c.msum_src_d = upload_vec(c.ar, c.msum_src_h);
  // Precision: the chain products run in the context's precision (FP32 in
  // precision 1).  The contractions of the mean fields and density matrices use
  // the compensated split (about 1e-13 relative) whenever a split mode is chosen:
  // the regularised inverse of rho scales mean-field errors by up to 1/eps_rho.
  for (auto& b : c.chains_full) {
    b.prec = c.precision;
    b.finalize(c.ar);
  }
  for (auto& b : c.chains) {
    b.prec = c.precision;
    b.finalize(c.ar);
  }
  c.gprods.prec = c.precision;
  c.gprods.finalize(c.ar);
  c.holes.prec = c.mf_hole_prec;
  c.holes.finalize(c.ar);
  // density matrices: compensated split FP32 (~1e-13 relative) in the split modes
  c.rho_holes.prec = c.hole_prec;
  c.rho_holes.finalize(c.ar);
  for (auto& hr : rrefs) c.red.add_term(hr.target, c.rho_holes.h[hr.hole], hr.alpha);
  for (auto& hr : hrefs) c.red.add_term(hr.target, c.holes.h[hr.hole], hr.alpha, hr.conjT);
  c.red.finalize(c.ar);

  // regularised inverse of rho times the mean fields (Calc_rhom1MF, gmctdh_objects.f90:1147-1194)
  for (int m : c.modes_dvr) {
    std::vector<int> states;
    if (c.multiset[m]) for (int s = 0; s < c.nstates; ++s) states.push_back(s);
    else states.push_back(0);
    for (int s : states) {
      RegInvDesc rd;
      memset(&rd, 0, sizeof(rd));
      rd.A = c.multiset[m] ? c.rho[m][s] : c.rho_ave[m];
      rd.n = c.m_of(m, s);
      rd.regtype = 0;
      rd.eps = c.eps_rho;
      if (!c.reginv_cold) {
        rd.vprev = c.ar.calloc_c((long long)rd.n * rd.n);
        rd.vcount = reinterpret_cast<int*>(c.ar.calloc_c(1));
        CK(cudaMemset(rd.vcount, 0, sizeof(int)));   // no warm start before the first call
      }
      rd.op_first = (int)c.mfop_h.size();
      for (int k = 0; k < c.noper[m]; ++k) {
        if (c.is_identity[m + f * k] || !c.ham_op[m][k]) continue;
        if (c.multiset[m] && c.oper[m][k][0] != s) continue;
        MFOp op;
        memset(&op, 0, sizeof(op));
        op.mf = c.mf[m][k];
        op.out = c.rhom1mf[m][k];
        op.n2 = c.m_of(m, c.oper[m][k][1]);
        c.mfop_h.push_back(op);
      }
      rd.op_count = (int)c.mfop_h.size() - rd.op_first;
      c.reg_h.push_back(rd);
    }
  }
  c.reg_d = upload_vec(c.ar, c.reg_h);
  c.mfop_d = upload_vec(c.ar, c.mfop_h);

  // SPF derivatives (derivatives.f90:96-153)
  size_t ssmem = 0;
  for (int m : c.modes_dvr) {
    std::vector<int> states;
    if (c.multiset[m]) for (int s = 0; s < c.nstates; ++s) states.push_back(s);
    else states.push_back(0);
    for (int s : states) {
      SpfDesc sd;
      memset(&sd, 0, sizeof(sd));
      sd.phi = c.d_in + c.naconftot + c.ipsi[m + f * s];
      sd.out_offset = c.naconftot + c.ipsi[m + f * s];
      sd.G = c.gmode[m];
      sd.n = c.m_of(m, s);
      sd.op_first = (int)c.spfop_h.size();
      for (int k = 0; k < c.noper[m]; ++k) {
        if (c.is_identity[m + f * k] || !c.ham_op[m][k]) continue;
        if (c.multiset[m] && c.oper[m][k][0] != s) continue;
        SpfOp op;
        memset(&op, 0, sizeof(op));
        op.ophi = c.ophi[m][k];
        op.rm = c.rhom1mf[m][k];
        op.n2 = c.m_of(m, c.oper[m][k][1]);
        c.spfop_h.push_back(op);
      }
      sd.op_count = (int)c.spfop_h.size() - sd.op_first;
      sd.ntile = (sd.G + SPF_TILE - 1) / SPF_TILE;
      sd.block_start = c.spf_tiles;
      c.spf_tiles += sd.ntile;
      sd.partial = c.ar.calloc_c((long long)sd.ntile * 2 * sd.n * sd.n);
      sd.X = c.ar.calloc_c((long long)sd.n * sd.n);
      c.spf_h.push_back(sd);
      ssmem = std::max(ssmem, sizeof(cplx) * (size_t)(2 * sd.G * sd.n));
    }
  }
  c.spf_smem = ssmem;
  c.spf_d = upload_vec(c.ar, c.spf_h);
  for (auto& x : c.spf_h) c.spf_nf = std::max(c.spf_nf, x.n);
  for (auto& x : c.spfop_h) c.spf_nf = std::max(c.spf_nf, x.n2);
  c.spfop_d = upload_vec(c.ar, c.spfop_h);

  // dA = f * sum_t ae_t * (H_t A)   (conjugate of Adot_tmp, gmctdh_objects.f90:578; derivatives.f90:155-156)
  for (int s = 0; s < c.nstates; ++s) {
    SumRange r;
    r.offset = c.aoff[s];
    r.n = c.naconf[s];
    r.first = (int)c.src_h.size();
    r.count = (int)srcs[s].size();
    for (auto& x : srcs[s]) c.src_h.push_back(x);
    c.sum_h.push_back(r);
  }
  c.sum_d = upload_vec(c.ar, c.sum_h);
  split_coeffs(c.src_h);
  c.src_d = upload_vec(c.ar, c.src_h);
  for (auto& b : c.gwp_rho_chain) b.finalize(c.ar);
  if (!c.modes_gwp.empty()) plan_gwp_derivs(c);
}

// Gaussian-parameter derivatives and the coefficient correction for Gaussian
// modes (derivatives.f90:158-236): Calc_CY per (mode, state) block, the
// Tikhonov solve, tau, then dA = S^-1 x_m (f H A) - tau x_m A over the Gaussian
// modes.  All FP64.
void plan_gwp_derivs(Ctx& c) {
  const int f = c.nmodes;
  const int ng = (int)c.modes_gwp.size();
  c.tau.assign(ng, std::vector<cplx*>(c.nstates, nullptr));
  for (int i = 0; i < ng; ++i) {
    const int m = c.modes_gwp[i];
    const double* a = c.gwpa_d + (size_t)c.gwp_lda * c.ns00max * i;
    const int nsets = c.multiset[m] ? c.nstates : 1;
    for (int s = 0; s < nsets; ++s) {
      const int n = c.m_of(m, s), nmd = c.nmodedof[m];
      const int nG = n * nmd;
      GwpCYDesc d;
      memset(&d, 0, sizeof(d));
      d.xi = psi_block(c, c.d_in, m, s);
      d.a = a;
      d.S = c.s00[i][s][s];
      d.Sm1 = c.s00m1[i][s];
      d.rho = c.multiset[m] ? c.rho[m][s] : c.rho_ave[m];
      d.Sa0 = c.ar.calloc_c((long long)nG * n);
      d.Sa0Sm1 = c.ar.calloc_c((long long)nG * n);
      d.M = c.ar.calloc_c(2LL * nG * (nG + 1));
      d.R = c.ar.calloc_c((long long)nG * nG);
      d.x = c.ar.calloc_c(nG);
      d.dxi_offset = c.naconftot + c.ipsi[m + f * s];
      c.tau[i][s] = c.ar.calloc_c((long long)n * n);
      d.tau = c.tau[i][s];
      d.nmd = nmd;
      d.lda = c.gwp_lda;
      d.n = n;
      d.nG = nG;
      d.eps = c.eps_C;
      d.op_first = (int)c.yop_h.size();
      for (int k = 0; k < c.noper[m]; ++k) {
        if (c.is_identity[m + f * k] || !c.ham_op[m][k]) continue;
        const int l = c.oper[m][k][0], r = c.oper[m][k][1];
        if (c.multiset[m] && l != s) continue;
        GwpYOp op;
        memset(&op, 0, sizeof(op));
        op.xi2 = psi_block(c, c.d_in, m, r);
        op.S12 = c.s00[i][s][set_of(c, m, r)];
        op.h = c.hmat[m][k];
        op.mf = c.mf[m][k];
        op.n2 = c.m_of(m, r);
        for (int q = 0; q < nmd; ++q) op.ops[q] = c.oper[m][k][2 + q];
        c.yop_h.push_back(op);
      }
      d.op_count = (int)c.yop_h.size() - d.op_first;
      c.cy_maxops = std::max(c.cy_maxops, d.op_count);
      c.cy_maxG = std::max(c.cy_maxG, nG);
      c.cy_maxn = std::max(c.cy_maxn, n);
      if (nG > 512) throw StatusError(MCTDH_EUNSUPPORTED, "Gaussian parameter system above 512 unknowns");
      c.cy_h.push_back(d);
    }
  }
  c.cy_d = upload_vec(c.ar, c.cy_h);
  c.yop_d = upload_vec(c.ar, c.yop_h);
  c.cy_part = c.ar.calloc_c((long long)c.cy_h.size() * c.cy_maxG * c.cy_maxn * std::max(c.cy_maxops, 1));
  // dA = S^-1 (f H A) - tau A on the Gaussian modes
  c.d_adot = c.ar.calloc_c(c.naconftot);
  c.d_dA = c.ar.calloc_c(c.naconftot);
  c.gwp_sinv.assign(ng, ProdBatch());
  c.gwp_tau.assign(ng, ProdBatch());
  for (int s = 0; s < c.nstates; ++s) {
    std::vector<int> sh = c.shape_of(s);
    const cplx* cur = c.d_adot + c.aoff[s];
    for (int i = 0; i < ng; ++i) {
      const int m = c.modes_gwp[i];
      cplx* out = (i + 1 == ng) ? c.d_dA + c.aoff[s] : c.ar.calloc_c(c.naconf[s]);
      c.gwp_sinv[i].add(cur, out, c.s00m1[i][set_of(c, m, s)], sh[m], 0, sh, m, sh[m], mkc(1, 0), 0);
      cur = out;
    }
    for (int i = 0; i < ng; ++i) {
      const int m = c.modes_gwp[i];
      c.gwp_tau[i].add(c.d_in + c.aoff[s], c.d_dA + c.aoff[s], c.tau[i][set_of(c, m, s)], sh[m], 0, sh, m, sh[m],
                       mkc(-1, 0), 1);
    }
  }
  for (auto& b : c.gwp_sinv) b.finalize(c.ar);
  for (auto& b : c.gwp_tau) b.finalize(c.ar);
}

// H_B * B for the CMF2 Lanczos (Calc_DHD_B, cmf2_derivatives.f90:1-80): chains over
// the non-identity operators of each term (grid modes, then Gaussian modes with
// D^H h D), no der_factor.
void plan_hb(Ctx& c) {
  const int f = c.nmodes;
  c.hb_chains.assign(f + 1, ProdBatch());
  c.dhd.assign(c.modes_gwp.size(), {});
  for (size_t i = 0; i < c.modes_gwp.size(); ++i) {
    const int m = c.modes_gwp[i];
    c.dhd[i].assign(c.noper[m], nullptr);
    for (int k = 0; k < c.noper[m]; ++k) {
      if (c.is_identity[m + f * k] || !c.ham_op[m][k]) continue;
      c.dhd[i][k] = c.ar.calloc_c((long long)c.m_of(m, c.oper[m][k][0]) * c.m_of(m, c.oper[m][k][1]));
    }
  }
  std::vector<std::vector<SumSrc>> srcs(c.nstates);
  // FP32 products keep complex FP32 intermediates; compensated ones the split pairs
  const int chain_fmt = c.hb_prec == 1 ? TF_F32 : (c.hb_prec ? TF_SPLIT : TF_C64);
  // FP32 products read the Krylov vector once converted to complex FP32 (8-byte
  // elements: state offsets count float2)
  const int hb_in_fmt = c.hb_prec == 1 ? TF_F32 : TF_C64;
  auto hb_in_at = [&](int s) -> cplx* {
    if (hb_in_fmt == TF_F32) return reinterpret_cast<cplx*>(reinterpret_cast<float2*>(c.d_hbin32) + c.aoff[s]);
    return c.d_hbin + c.aoff[s];
  };
  // The general terms of one state pair share products: each pair's chains form a
  // prefix tree over the modes, with the modes on which all of the pair's terms
  // carry the same matrix first (the SPF overlaps between two state sets, for
  // example), so a product common to several terms is computed once.  The order
  // of the mode products changes only the rounding; a pair with one term keeps the
  // reference order (grid modes, then Gaussian modes with D^H h D).
  std::vector<int> base_order = c.modes_dvr;
  base_order.insert(base_order.end(), c.modes_gwp.begin(), c.modes_gwp.end());
  auto hb_mat = [&](int t, int m) -> const cplx* {
    const int k = c.ioper[m + f * t];
    if (c.is_identity[m + f * k]) return nullptr;   // identity; D^H S D = 1 on Gaussian modes
    return c.is_gwp[m] ? c.dhd[c.gwp_of[m]][k] : c.hmat[m][k];
  };
  std::map<std::pair<int, int>, std::vector<int>> pair_terms;
  for (int t : c.general_terms) pair_terms[std::make_pair(c.lhs[t], c.rhs[t])].push_back(t);
  for (auto& pt : pair_terms) {
    const int s1 = pt.first.first, s2 = pt.first.second;
    const std::vector<int>& terms = pt.second;
    std::vector<int> order = base_order;
    std::vector<int> distinct(f, 0);
    for (int m : order) {
      std::set<const cplx*> mats;
      for (int t : terms) mats.insert(hb_mat(t, m));
      distinct[m] = (int)mats.size();
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return distinct[a] < distinct[b]; });
    struct Node {
      TRef ref;
      int depth;
    };
    std::vector<Node> nodes(1);
    nodes[0].ref.p = hb_in_at(s2);
    nodes[0].ref.fmt = hb_in_fmt;
    nodes[0].ref.shape = c.shape_of(s2);
    nodes[0].depth = 0;
    std::map<std::tuple<int, int, const cplx*>, int> child;   // (node, mode, matrix) -> node
    for (int t : terms) {
      int cur = 0;
      for (int m : order) {
        const cplx* mat = hb_mat(t, m);
        if (!mat) continue;
        const auto key = std::make_tuple(cur, m, mat);
        auto it = child.find(key);
        if (it != child.end()) {
          cur = it->second;
          continue;
        }
        const int n1 = c.m_of(m, s1);
        Node nd;
        nd.ref.shape = nodes[cur].ref.shape;
        nd.ref.shape[m] = n1;
        nd.ref.p = c.ar.calloc_c(prod_range(nd.ref.shape, 0, (int)nd.ref.shape.size()));
        nd.ref.fmt = chain_fmt;
        nd.depth = nodes[cur].depth + 1;
        c.hb_chains[nd.depth].add(nodes[cur].ref.p, nd.ref.p, mat, n1, 0, nodes[cur].ref.shape, m, n1, mkc(1, 0), 0,
                                  nodes[cur].ref.fmt, chain_fmt);
        nodes.push_back(nd);
        child[key] = (int)nodes.size() - 1;
        cur = (int)nodes.size() - 1;
      }
      srcs[s1].push_back(SumSrc{nodes[cur].ref.p, c.ae[t], nodes[cur].ref.fmt});
    }
  }
  for (auto& kv : c.gmat) {
    const int s = kv.first.first, m = kv.first.second;
    const int n = c.m_of(m, s);
    std::vector<int> sh = c.shape_of(s);
    cplx* out = c.ar.calloc_c(prod_range(sh, 0, (int)sh.size()));
    c.hb_chains[1].add(hb_in_at(s), out, kv.second, n, 0, sh, m, n, mkc(1, 0), 0, hb_in_fmt, chain_fmt);
    srcs[s].push_back(SumSrc{out, mkc(1, 0), chain_fmt});
  }
  for (int s = 0; s < c.nstates; ++s)
    if (c.c0[s].x != 0.0 || c.c0[s].y != 0.0) srcs[s].push_back(SumSrc{c.d_hbin + c.aoff[s], c.c0[s]});
  for (auto& b : c.hb_chains) {
    b.prec = c.hb_prec;   // H_B * B feeds the Lanczos recurrence, which stays FP64
    b.finalize(c.ar);
  }
  std::vector<SumRange> ranges;
  for (int s = 0; s < c.nstates; ++s) {
    SumRange r;
    r.offset = c.aoff[s];
    r.n = c.naconf[s];
    r.first = (int)c.hbsrc_h.size();
    r.count = (int)srcs[s].size();
    for (auto& x : srcs[s]) c.hbsrc_h.push_back(x);
    ranges.push_back(r);
  }
  c.hbsum_d = upload_vec(c.ar, ranges);
  split_coeffs(c.hbsrc_h);
  c.hbsrc_d = upload_vec(c.ar, c.hbsrc_h);
}

// Overlap plan between states y1 and y2: o11 = <1|1>, o22 = <2|2>, o12 = <1|2>
// (norm_wf / WF_Ovl / DeltaPsi, gmctdh_objects.f90:21-226).  prec 2: the mode
// products of the chains in compensated split FP32 (~1e-13 relative); used for
// the step-error norm DeltaPsi of split-precision contexts, where 1 - Re<1|2>/..
// is of order eps_int^2 / 2 >> 1e-13.  Norms and C(t) keep prec 0.
void plan_ovl(Ctx& c, OvlPlan& P, cplx* y1, cplx* y2, int prec, bool norm_only, bool shared) {
  const int f = c.nmodes;
  P.npk = c.npk;
  P.d_result = c.ar.calloc_c(3 * c.npk);
  struct Smat { cplx* s11; cplx* s22; cplx* s12; };
  std::vector<std::vector<Smat>> S(f, std::vector<Smat>(c.nstates));
  std::vector<HoleRef> hrefs;
  for (int m : c.modes_dvr) {
    for (int s = 0; s < c.nstates; ++s) {
      if (!c.multiset[m] && s > 0) { S[m][s] = S[m][0]; continue; }
      const int n = c.m_of(m, s);
      const long long G = c.gmode[m];
      cplx* p1 = y1 + c.naconftot + c.ipsi[m + f * s];
      cplx* p2 = y2 + c.naconftot + c.ipsi[m + f * s];
      Smat sm;
      sm.s11 = c.ar.calloc_c((long long)n * n);
      sm.s22 = c.ar.calloc_c((long long)n * n);
      sm.s12 = c.ar.calloc_c((long long)n * n);
      int h11 = P.spf_holes.add(c.ar, p1, p1, G, 1, n, n);
      int h22 = P.spf_holes.add(c.ar, p2, p2, G, 1, n, n);
      int h12 = P.spf_holes.add(c.ar, p1, p2, G, 1, n, n);
      hrefs.push_back(HoleRef{h11, P.spf_red.add_target(sm.s11, n, n, n, 1), mkc(1, 0)});
      hrefs.push_back(HoleRef{h22, P.spf_red.add_target(sm.s22, n, n, n, 1), mkc(1, 0)});
      hrefs.push_back(HoleRef{h12, P.spf_red.add_target(sm.s12, n, n, n, 0), mkc(1, 0)});
      S[m][s] = sm;
    }
  }
  // Gaussian modes: normalised Gaussian overlaps; <1|1> and <2|2> from the upper
  // triangle with unit diagonal (gmctdh_objects.f90:21-97), <1|2> in full (:101-180)
  for (int m : c.modes_gwp) {
    const int i = c.gwp_of[m];
    const double* a = c.gwpa_d + (size_t)c.gwp_lda * c.ns00max * i;
    for (int s = 0; s < c.nstates; ++s) {
      if (!c.multiset[m] && s > 0) { S[m][s] = S[m][0]; continue; }
      const int n = c.m_of(m, s);
      Smat sm;
      cplx* outs[3];
      for (int q = 0; q < 3; ++q) outs[q] = c.ar.calloc_c((long long)n * n);
      sm.s11 = outs[0];
      sm.s22 = outs[1];
      sm.s12 = outs[2];
      const cplx* p1 = psi_block(c, y1, m, s);
      const cplx* p2 = psi_block(c, y2, m, s);
      const cplx* L[3] = {p1, p2, p1};
      const cplx* Rr[3] = {p1, p2, p2};
      for (int q = 0; q < 3; ++q) {
        GwpOvlDesc d;
        memset(&d, 0, sizeof(d));
        d.xi1 = L[q];
        d.xi2 = Rr[q];
        d.a = a;
        d.out = outs[q];
        d.nmd = c.nmodedof[m];
        d.lda = c.gwp_lda;
        d.n1 = n;
        d.n2 = n;
        d.kind = (q < 2) ? 0 : 1;
        P.gwp_h.push_back(d);
      }
      S[m][s] = sm;
    }
  }
  P.gwp_d = upload_vec(c.ar, P.gwp_h);
  // the SPF overlaps over the grid: compensated split FP32 (~1e-13) where the
  // plan's chains are (the step-error overlaps of the split paths), else FP64
  P.spf_holes.prec = prec;
  P.spf_holes.finalize(c.ar);
  for (auto& hr : hrefs) P.spf_red.add_term(hr.target, P.spf_holes.h[hr.hole], hr.alpha);
  P.spf_red.finalize(c.ar);
  std::vector<int> order = c.modes_dvr;
  order.insert(order.end(), c.modes_gwp.begin(), c.modes_gwp.end());
  P.chain.assign(order.size() + 1, ProdBatch());
  std::vector<HoleRef> drefs;
  // per packet W: results 3W + {0, 1, 2}
  std::vector<int> tgt(3 * c.npk);
  for (int q = 0; q < 3 * c.npk; ++q) tgt[q] = P.dot_red.add_target(P.d_result + q, 1, 1, 1, 0);
  for (int s = 0; s < c.nstates; ++s) {
    std::vector<int> sh = c.shape_of(s);
    const long long N = c.naconf[s];
    cplx* a1 = y1 + c.aoff[s];
    cplx* a2 = y2 + c.aoff[s];
    cplx* cur[3] = {a1, a2, a2};
    int curfmt[3] = {TF_C64, TF_C64, TF_C64};
    const int cfmt = prec ? TF_SPLIT : TF_C64;
    // each chain alternates between two buffers (depth i reads i - 1's output);
    // plans run on the context stream share them (c.ovl_pool: one plan runs at a
    // time), the CMF2 error overlap, which runs beside other work, has its own
    cplx* pp[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    if (shared)
      for (int q = 0; q < 3; ++q)
        for (int par = 0; par < 2; ++par) pp[q][par] = c.ovl_pool[std::make_tuple(s, q, par)];
    for (size_t i = 0; i < order.size(); ++i) {
      const int m = order[i];
      const int n = sh[m];
      cplx* mats[3] = {S[m][s].s11, S[m][s].s22, S[m][s].s12};
      for (int q = 0; q < (norm_only ? 1 : 3); ++q) {
        cplx*& buf = pp[q][i & 1];
        if (!buf) {
          buf = c.ar.calloc_c(N);
          if (shared) c.ovl_pool[std::make_tuple(s, q, (int)(i & 1))] = buf;
        }
        cplx* out = buf;
        P.chain[i + 1].add(cur[q], out, mats[q], n, 0, sh, m, n, mkc(1, 0), 0, curfmt[q], cfmt);
        cur[q] = out;
        curfmt[q] = cfmt;
      }
    }
    const long long n1 = c.n1[s];
    for (int w = 0; w < c.npk; ++w) {
      const long long o = n1 * w;
      drefs.push_back(HoleRef{P.dots.add(c.ar, a1 + o, cur[0] + o, n1, 1, 1, 1, TF_C64, curfmt[0]), tgt[3 * w],
                              mkc(1, 0)});
      if (norm_only) continue;
      drefs.push_back(HoleRef{P.dots.add(c.ar, a2 + o, cur[1] + o, n1, 1, 1, 1, TF_C64, curfmt[1]), tgt[3 * w + 1],
                              mkc(1, 0)});
      drefs.push_back(HoleRef{P.dots.add(c.ar, a1 + o, cur[2] + o, n1, 1, 1, 1, TF_C64, curfmt[2]), tgt[3 * w + 2],
                              mkc(1, 0)});
    }
  }
  for (auto& b : P.chain) {
    b.prec = prec;
    b.finalize(c.ar);
  }
  P.dots.finalize(c.ar);
  for (auto& hr : drefs) P.dot_red.add_term(hr.target, P.dots.h[hr.hole], hr.alpha);
  P.dot_red.finalize(c.ar);
}

// ---------------------------------------------------------------------------
// Execution
// ---------------------------------------------------------------------------
cudaEvent_t take_event(Ctx& c) {
  if (!c.evpool.empty()) {
    cudaEvent_t e = c.evpool.back();
    c.evpool.pop_back();
    return e;
  }
  cudaEvent_t e;
  CK(cudaEventCreate(&e));
  return e;
}
// Bracket one launch with events when profiling (on the context stream).
struct ProfScope {
  Ctx& c;
  int kid;
  double flops, bytes;
  cudaEvent_t a = nullptr;
  ProfScope(Ctx& cc, int k, double f = 0, double b = 0) : c(cc), kid(k), flops(f), bytes(b) {
    if (c.profiling) {
      a = take_event(c);
      CK(cudaEventRecord(a, c.st));
    }
  }
  ~ProfScope() {
    if (c.profiling && a) {
      cudaEvent_t b = take_event(c);
      cudaEventRecord(b, c.st);
      c.pending.push_back(PendingEv{kid, a, b, flops, bytes});
    }
  }
};
// Routine timers: RT_* are the reference's timer numbers minus one.
enum { RT_CALCDERIVS, RT_OVL, RT_MEANFIELD, RT_CY, RT_H1MODE, RT_SPF_DVR, RT_SPF_GWP, RT_LANCZOS };
struct RtScope {
  Ctx& c;
  int id;
  bool call;
  cudaEvent_t a = nullptr;
  RtScope(Ctx& cc, int i, bool counts_call = true, bool on = true) : c(cc), id(i), call(counts_call) {
    if (c.timing && on) {
      a = take_event(c);
      CK(cudaEventRecord(a, c.st));
    }
  }
  ~RtScope() {
    if (c.timing && a) {
      cudaEvent_t b = take_event(c);
      cudaEventRecord(b, c.st);
      c.rt_pending.push_back(Ctx::RtEv{id, a, b, call});
    }
  }
};
void drain_timing(Ctx& c) {
  if (c.rt_pending.empty()) return;
  CK(cudaDeviceSynchronize());
  for (auto& p : c.rt_pending) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, p.a, p.b));
    c.rt_ms[p.id] += ms;
    if (p.call) c.rt_calls[p.id] += 1;
    c.evpool.push_back(p.a);
    c.evpool.push_back(p.b);
  }
  c.rt_pending.clear();
}

void drain_profile(Ctx& c) {
  if (c.pending.empty()) return;
  CK(cudaStreamSynchronize(c.st));
  for (auto& p : c.pending) {
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, p.a, p.b));
    KProf& k = c.prof[p.kid];
    k.ms += ms;
    k.launches += 1;
    k.flops += p.flops;
    k.bytes += p.bytes;
    c.evpool.push_back(p.a);
    c.evpool.push_back(p.b);
  }
  c.pending.clear();
}

// Run `body` (a launch sequence without host synchronisation) through a CUDA
// graph captured on its first use for this (kind, key); if capture is not
// possible the sequence is launched directly from then on.
template <typename F>
void run_graphed(Ctx& c, int kind, const void* key, F&& body) {
  if (c.profiling || c.graphs_off || c.timing) {
    body();
    return;
  }
  auto k = std::make_pair(kind, key);
  auto it = c.graphs.find(k);
  if (it == c.graphs.end()) {
    if (!c.graph_seen.count(k)) {
      // first use runs directly: lazily built plans allocate then, never under capture
      c.graph_seen.insert(k);
      body();
      return;
    }
    const long long l0 = c.launches, e0 = c.eom_count, h0 = c.hb_count;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      c.graphs_off = true;
      body();
      return;
    }
    bool ok = true;
    try {
      body();
    } catch (...) {
      ok = false;
    }
    cudaError_t e = cudaStreamEndCapture(c.st, &g);
    cudaGraphExec_t ge = nullptr;
    if (ok && e == cudaSuccess && g) ok = (cudaGraphInstantiate(&ge, g, 0) == cudaSuccess);
    else ok = false;
    if (g) cudaGraphDestroy(g);
    const long long nl = c.launches - l0, ne = c.eom_count - e0, nh = c.hb_count - h0;
    c.launches = l0;
    c.eom_count = e0;
    c.hb_count = h0;
    if (!ok) {
      cudaGetLastError();
      c.graphs_off = true;
      body();
      return;
    }
    it = c.graphs.emplace(k, Ctx::GraphRec{ge, nl, ne, nh}).first;
  }
  CK(cudaGraphLaunch(it->second.exec, c.st));
  c.launches += it->second.launches;
  c.eom_count += it->second.eoms;
  c.hb_count += it->second.hbs;
}

// Issue the enclosed launches on another stream of the context (the launch
// helpers all use c.st).
struct StreamSwap {
  Ctx& c;
  cudaStream_t old;
  StreamSwap(Ctx& ctx, cudaStream_t s) : c(ctx), old(ctx.st) { c.st = s; }
  ~StreamSwap() { c.st = old; }
};

void run_prod(Ctx& c, const ProdBatch& b) {
  if (b.h.empty()) return;
  ProfScope ps(c, KP_PROD, b.flops, b.bytes);
  launch_prod(b.d, (int)b.h.size(), b.nblocks, b.maxn, c.st, b.prec);
  c.count();
}
void run_hole(Ctx& c, const HoleBatch& b) {
  if (b.h.empty()) return;
  ProfScope ps(c, KP_HOLE, b.flops, b.bytes);
  launch_hole(b.d, (int)b.h.size(), b.nblocks, c.st, b.prec);
  c.count();
}
void run_red(Ctx& c, const RedBatch& b) {
  if (b.tg.empty()) return;
  ProfScope ps(c, KP_RED);
  launch_reduce(b.d_tg, (int)b.tg.size(), b.d_terms, c.st);
  c.count();
}

// Gaussian modes, first part of the EOM: S00, S00^-1 (tikh) and h1mode.
void gwp_setup_run(Ctx& c) {
  ProfScope ps(c, KP_GWP);
  launch_gwp_ovl(c.gs_d, (int)c.gs_h.size(), c.st);
  launch_tikh_inv(c.gsreg_d, (int)c.gsreg_h.size(), c.st);
  launch_gwp_h1(c.gh1_d, (int)c.gh1_h.size(), c.st);
  c.count(3);
}

// Gaussian modes, last part: parameter derivatives into out's psi part and the
// corrected dA into out's coefficient part (from d_adot).
// Calc_CY and the Tikhonov parameter solve: der_factor * x into out's psi part, tau
void gwp_solve_run(Ctx& c, cplx* out) {
  RtScope rt(c, RT_CY);   // Calc_CY and the parameter solve (gmctdh_objects.f90:1198-1333)
  ProfScope ps(c, KP_GWP);
  launch_gwp_cy(c.cy_d, (int)c.cy_h.size(), c.cy_maxG, c.cy_maxn, c.cy_maxops, c.yop_d, c.cy_part, c.st);
  launch_gwp_solve(c.cy_d, (int)c.cy_h.size(), c.cy_maxG, c.der, out, c.d_status, c.st);
  c.count(6 + (c.cy_maxG + GWP_QR_PW - 1) / GWP_QR_PW);
}

void gwp_derivs_run(Ctx& c, cplx* out) {
  RtScope rt(c, RT_SPF_GWP);
  gwp_solve_run(c, out);
  for (auto& b : c.gwp_sinv) run_prod(c, b);
  for (auto& b : c.gwp_tau) run_prod(c, b);
  CK(cudaMemcpyAsync(out, c.d_dA, sizeof(cplx) * c.naconftot, cudaMemcpyDeviceToDevice, c.st));
}

// EOM on d_in -> out (full vector [dA | dpsi]).  mf_only: only the operator
// matrices, density matrices, mean fields and rho^-1 MF that CMF2 consumes
// (cmf2_base.f90:78-87, 122-130); the coefficient and SPF derivatives are skipped.
void run_reginv(Ctx& c) {
  ProfScope ps(c, KP_REGINV);
  launch_reginv(c.reg_d, (int)c.reg_h.size(), c.mfop_d, c.d_status, c.st);
  c.count();
}

// The packet stage of the EOM (plan_packets).
void run_packets(Ctx& c) {
  ProfScope ps(c, KP_TERMSUM);
  if (c.pk_sum2.n) {
    launch_termsum(c.pk_xa, c.pk_sum2.ranges, c.pk_sum2.n, c.pk_sum2.srcs, c.naconftot, c.st, c.precision);
    c.count();
  }
  for (int k = 0; k < c.ndiss1; ++k) {
    const Ctx::SumPlan& sp = c.pk_sum1[k];
    launch_termsum(c.pk_va + (long long)k * c.naconftot, sp.ranges, sp.n, sp.srcs, c.naconftot, c.st, c.precision);
    c.count();
  }
  if (c.npk > 1) run_ovl(c, c.pk_norm);
  launch_pk_gram(c.pk_pairs, c.pk_npairs, c.pk_st, c.nstates, c.pk_partial, c.st);
  launch_pk_coef(c.pk_args, c.st);
  c.count(2);
  if (c.pk_nmix) {
    launch_pk_mix(c.pk_mix, c.pk_nmix, c.pk_st, c.nstates, c.n1tot, c.npk, nullptr, c.st);
    c.count();
  }
  for (auto& b : c.aux_chains) run_prod(c, b);
  run_hole(c, c.aux_holes);
  run_red(c, c.aux_red);
}

void eom(Ctx& c, cplx* out, bool mf_only = false, bool reginv = true) {
  RtScope rt_all(c, RT_CALCDERIVS, true, !mf_only);   // derivatives.f90:92-476
  const bool gwp = !c.modes_gwp.empty();
  if (gwp) gwp_setup_run(c);
  if (c.d_in32) {
    launch_to_f32(c.d_in32, c.d_in, c.naconftot, c.st);
    c.count();
  }
  if (c.d_insplit) {
    launch_to_split(c.d_insplit, c.d_in, c.naconftot, c.st);
    c.count();
  }
  {
    RtScope rt(c, RT_H1MODE);
    ProfScope ps(c, KP_H1);
    launch_h1(c.h1_d, (int)c.h1_h.size(), c.h1_maxn2, c.h1_smem, true, c.st, c.precision);
    launch_matsum(c.msum_d, (int)c.msum_h.size(), c.msum_src_d, c.st);
    c.count(3);
  }
  RtScope rt_mf(c, RT_MEANFIELD);   // gmctdh_objects.f90:511-1140
  // the deepest level holds only the full products H_t A of the right chains (dA)
  const size_t depth_end = mf_only ? c.chains.size() - 1 : c.chains.size();
  for (size_t i = 1; i < depth_end; ++i) run_prod(c, c.chains[i]);
  if (!mf_only)
    for (size_t i = 1; i < c.chains_full.size(); ++i) run_prod(c, c.chains_full[i]);
  if (!mf_only) run_prod(c, c.gprods);
  for (auto& b : c.gwp_rho_chain) run_prod(c, b);
  run_hole(c, c.rho_holes);
  run_hole(c, c.holes);
  run_red(c, c.red);
  if (c.pk_on) run_packets(c);
  if (reginv || !mf_only) run_reginv(c);
  if (mf_only) {
    c.eom_count++;
    return;
  }
  {
    ProfScope ps(c, KP_TERMSUM, 0.0, 16.0 * (double)c.src_h.size() * (double)c.naconftot / std::max(1, c.nstates));
    launch_termsum(gwp ? c.d_adot : out, c.sum_d, (int)c.sum_h.size(), c.src_d, c.naconftot, c.st, c.precision);
    c.count();
  }
  {
    RtScope rt(c, RT_SPF_DVR);
    ProfScope ps(c, KP_SPF);
    launch_spf(c.spf_d, (int)c.spf_h.size(), c.spf_tiles, c.spfop_d, out, c.der, c.d_status, c.st, c.precision, c.spf_nf);
    c.count(3);
  }
  if (gwp) gwp_derivs_run(c, out);
  // Lagrange multipliers: dA += A (multLagDiag I + i multLag) (derivatives.f90:238-242)
  if (c.pk_mult && !c.skip_mult) {
    launch_pk_mix(c.pk_mult, 1, c.pk_st, c.nstates, c.n1tot, c.npk, out, c.st);
    c.count();
  }
  c.eom_count++;
}

void eom_from(Ctx& c, const cplx* y, cplx* out) {
  if (y != c.d_in) CK(cudaMemcpyAsync(c.d_in, y, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
  eom(c, out);
}

void run_ovl(Ctx& c, OvlPlan& P) {
  RtScope rt(c, RT_OVL);   // norm_wf / WF_Ovl / DeltaPsi
  if (!P.gwp_h.empty()) {
    launch_gwp_ovl(P.gwp_d, (int)P.gwp_h.size(), c.st);
    c.count();
  }
  run_hole(c, P.spf_holes);
  run_red(c, P.spf_red);
  for (auto& b : P.chain) run_prod(c, b);
  run_hole(c, P.dots);
  run_red(c, P.dot_red);
}

void check_status(Ctx& c) {
  int st = 0;
  CK(cudaMemcpyAsync(&st, c.d_status, sizeof(int), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  if (st != 0) {
    CK(cudaMemsetAsync(c.d_status, 0, sizeof(int), c.st));
    if (st & DEVST_EIG_NOCONV) throw StatusError(MCTDH_EEIG, "Jacobi eigensolver did not converge");
    if (st & DEVST_CHOL_FAIL) throw StatusError(MCTDH_EEIG, "SPF overlap matrix is not positive definite");
    throw StatusError(MCTDH_ENONFINITE, "device status " + std::to_string(st));
  }
}

// o11, o22, o12 summed over the packets (trace_wf, the autocorrelation of output.f90:143-149)
void read_ovl(Ctx& c, OvlPlan& P, cplx out[3]) {
  std::vector<cplx> v(3 * P.npk);
  CK(cudaMemcpyAsync(v.data(), P.d_result, sizeof(cplx) * v.size(), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  for (int q = 0; q < 3; ++q) {
    out[q] = mkc(0, 0);
    for (int w = 0; w < P.npk; ++w) out[q] = cadd(out[q], v[3 * w + q]);
  }
}

// DeltaPsi (gmctdh_objects.f90:206-248): sqrt|2 (1 - Re o12 / sqrt(o11 o22))| for one
// packet; sqrt(2 sum_W |sqrt(o11 o22) - Re o12| / sum_W sqrt(o11 o22)) for a mixture.
double ovl_delta(Ctx& c, OvlPlan& P) {
  std::vector<cplx> v(3 * P.npk);
  CK(cudaMemcpyAsync(v.data(), P.d_result, sizeof(cplx) * v.size(), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  if (P.npk == 1) return sqrt(fabs(2.0 * (1.0 - v[2].x / sqrt(v[0].x * v[1].x))));
  double num = 0.0, pop = 0.0;
  for (int w = 0; w < P.npk; ++w) {
    const double d = sqrt(v[3 * w].x * v[3 * w + 1].x);
    pop += d;
    num += fabs(d - v[3 * w + 2].x);
  }
  return sqrt(2.0 * num / pop);
}

// Cash-Karp and Dormand-Prince tableaux (integrator.f90:107-121, :171-185)
const double CK_A[6] = {0.0, 0.2, 0.3, 0.6, 1.0, 0.875};
const double CK_B[6][5] = {{0},
                           {0.2},
                           {0.075, 0.225},
                           {0.3, -0.9, 1.2},
                           {-11.0 / 54.0, 2.5, -70.0 / 27.0, 35.0 / 27.0},
                           {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0}};
const double CK_C[6] = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
const double CK_D[6] = {2825.0 / 27648.0, 0.0, 18575.0 / 48384.0, 13525.0 / 55296.0, 277.0 / 14336.0, 0.25};
const double DP_B[6][5] = {{0},
                           {0.2},
                           {0.075, 0.225},
                           {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0},
                           {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0},
                           {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0}};
const double DP_C[6] = {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0};
const double DP_D[7] = {5179.0 / 57600.0, 0.0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                        187.0 / 2100.0, 0.025};
const double RK_SAFETY = 0.9, RK_PGROW = -0.2, RK_PSHRNK = -0.25, RK_MINSCAL = 0.1, RK_MAXSCAL = 5.0;

// RK stage combination out = base + dt * sum_j coef_j k_j, with dt read from the
// device (c.d_scal[0]) so that a whole attempt can replay as one CUDA graph.
void stage(Ctx& c, cplx* out, const cplx* base, const double* coef, int nk, int kofs) {
  StageArgs a;
  memset(&a, 0, sizeof(a));
  int n = 0;
  for (int j = 0; j < nk; ++j) {
    if (coef[j] == 0.0) continue;
    a.k[n] = c.d_k[kofs + j];
    a.c[n] = coef[j];
    ++n;
  }
  a.nk = n;
  launch_ens_stage(out, base, a, c.d_scal, c.d_off1, 1, c.ntot, c.st);
  c.count();
}

// One rkck/rkdp attempt from d_y with k1 in d_k[0]; leaves the 5th-order state in
// d_tmp, the embedded state in d_err; returns errmax / eps (DeltaPsi).
double rk_attempt(Ctx& c, double t, double dt, int method) {
  (void)t;
  const bool dp = (method == 2);
  c.h_scal[0] = dt;
  CK(cudaMemcpyAsync(c.d_scal, c.h_scal, sizeof(double), cudaMemcpyHostToDevice, c.st));
  // the attempt is the same launch sequence every time: one CUDA graph per method
  run_graphed(c, 10 + method, nullptr, [&] {
    for (int st = 1; st < 6; ++st) {
      stage(c, c.d_in, c.d_y, dp ? DP_B[st] : CK_B[st], st, 0);
      eom(c, c.d_k[st]);
    }
    stage(c, c.d_tmp, c.d_y, dp ? DP_C : CK_C, 6, 0);
    if (dp) {
      CK(cudaMemcpyAsync(c.d_in, c.d_tmp, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
      eom(c, c.d_k[6]);
      stage(c, c.d_err, c.d_y, DP_D, 7, 0);
    } else {
      stage(c, c.d_err, c.d_y, CK_D, 6, 0);
    }
    run_ovl(c, c.dpsi_plan);
  });
  const double delta = ovl_delta(c, c.dpsi_plan);
  check_status(c);
  if (!std::isfinite(delta)) throw StatusError(MCTDH_ENONFINITE, "non-finite RK error estimate");
  return delta / c.eps_int;
}

// rkqs (integrator.f90:36-91) on d_y; d_k[0] holds dA/dpsi at t on entry.
void rkqs(Ctx& c, double t, double htry, double* hdid, double* hnext, int method, long long* attempts) {
  double dt = htry, errmax;
  const double errcon = pow(5.0 / RK_SAFETY, 1.0 / RK_PGROW);
  while (true) {
    ++*attempts;
    errmax = rk_attempt(c, t, dt, method);
    if (errmax < 1.0 || dt <= c.min_stepsize) break;
    dt = std::max(RK_MINSCAL * dt, RK_SAFETY * dt * pow(errmax, RK_PSHRNK));
    dt = std::max(dt, c.min_stepsize);
  }
  double hn = (errmax > errcon) ? RK_SAFETY * dt * pow(errmax, RK_PGROW) : dt * RK_MAXSCAL;
  hn = std::max(hn, c.min_stepsize);
  hn = std::min(hn, c.writetime);
  *hdid = dt;
  *hnext = hn;
  CK(cudaMemcpyAsync(c.d_y, c.d_tmp, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
  if (method == 2)
    CK(cudaMemcpyAsync(c.d_k[0], c.d_k[6], sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
}

// ---------------------------------------------------------------------------
// Adams PECE with variable step size (Adams, integrator.f90:244-380), on the
// resident state; the derivative at the current point is kept in ad_dcur.
// ---------------------------------------------------------------------------
void adams_plan(Ctx& c) {
  if (c.ad_planned) return;
  const int k = c.int_order;
  if (k < 1 || k > 6) throw StatusError(MCTDH_EUNSUPPORTED, "Adams order must be 1..6");
  for (int i = 0; i < k; ++i) c.ad_hist.push_back(c.ar.calloc_c(c.ntot));
  c.ad_hprev.assign(k, 0.0);
  c.ad_dcur = c.ar.calloc_c(c.ntot);
  c.ad_temp = c.ar.calloc_c(c.ntot);
  c.ad_new = c.ar.calloc_c(c.ntot);
  c.ad_new1 = c.ar.calloc_c(c.ntot);
  c.ad_dnew = c.ar.calloc_c(c.ntot);
  c.ad_d1 = c.ar.calloc_c(c.ntot);
  plan_ovl(c, c.ad_plan, c.ad_new, c.ad_new1, (c.precision && c.eps_int >= 1e-5) ? 2 : 0);
  c.ad_planned = true;
}

// Solve the n x n system M x = b (column-major, leading dimension ld) by Gaussian
// elimination with partial pivoting (the work of dgesv).
void small_solve(std::vector<double> M, int n, int ld, std::vector<double>& b) {
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (fabs(M[r + ld * col]) > fabs(M[piv + ld * col])) piv = r;
    if (M[piv + ld * col] == 0.0) throw StatusError(MCTDH_ESTEP, "singular Adams system");
    if (piv != col) {
      for (int j = 0; j < n; ++j) std::swap(M[col + ld * j], M[piv + ld * j]);
      std::swap(b[col], b[piv]);
    }
    for (int r = col + 1; r < n; ++r) {
      const double f = M[r + ld * col] / M[col + ld * col];
      for (int j = col; j < n; ++j) M[r + ld * j] -= f * M[col + ld * j];
      b[r] -= f * b[col];
    }
  }
  for (int r = n - 1; r >= 0; --r) {
    double v = b[r];
    for (int j = r + 1; j < n; ++j) v -= M[r + ld * j] * b[j];
    b[r] = v / M[r + ld * r];
  }
}

// out = base + w[0] dcur + sum_{i=1..nprev} w[i] hist[i-1]
void adams_combine(Ctx& c, cplx* out, const double* w, int nprev) {
  StageArgs a;
  memset(&a, 0, sizeof(a));
  a.k[0] = c.ad_dcur;
  a.c[0] = w[0];
  for (int i = 1; i <= nprev; ++i) {
    a.k[i] = c.ad_hist[i - 1];
    a.c[i] = w[i];
  }
  a.nk = nprev + 1;
  launch_stage(out, c.d_y, a, 1.0, c.ntot, c.st);
  c.count();
}
// out = base + w * d
void adams_axpy(Ctx& c, cplx* out, const cplx* base, const cplx* d, double w) {
  StageArgs a;
  memset(&a, 0, sizeof(a));
  a.k[0] = d;
  a.c[0] = w;
  a.nk = 1;
  launch_stage(out, base, a, 1.0, c.ntot, c.st);
  c.count();
}

void adams_step(Ctx& c, double t, double htry, double* hdid, double* hnext, long long* attempts) {
  const int k = c.int_order;
  const double minscal = 0.3, maxscal = 4.0, safety = 0.95;
  const double pow_shrink = -1.0 / (double)(k + 1);
  const int ld = k + 2;
  // M(j, i) = (x_(n-i) - x_n)^j for the columns i >= 1 (:259-268); column -1 per step size
  std::vector<double> M((size_t)ld * ld, 0.0);   // column index i + 1 for i = -1..k
  for (int i = 0; i < ld; ++i) M[0 + ld * i] = 1.0;
  double hsum = 0.0;
  for (int i = 1; i <= k; ++i) {
    hsum -= c.ad_hprev[i - 1];
    double d = hsum;
    for (int j = 1; j <= k + 1; ++j) {
      M[j + ld * (i + 1)] = d;
      d *= hsum;
    }
  }
  double dt = htry, errmax = 0.0;
  while (true) {
    ++*attempts;
    std::vector<double> B(ld);
    B[0] = dt;
    double d = dt;
    for (int j = 1; j <= k + 1; ++j) {
      M[j + ld * 0] = d;
      d *= dt;
      B[j] = d / (double)(j + 1);
    }
    // predictor (order k): columns 0..k-1
    std::vector<double> P((size_t)ld * ld, 0.0), xp(B.begin(), B.begin() + k);
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < k; ++i) P[j + ld * i] = M[j + ld * (i + 1)];
    small_solve(P, k, ld, xp);
    // correctors: order k+1 (columns -1..k-1) and order k+2 (columns -1..k)
    std::vector<double> x1(B.begin(), B.begin() + k + 1), x2(B.begin(), B.begin() + k + 2);
    std::vector<double> C1((size_t)ld * ld, 0.0), C2((size_t)ld * ld, 0.0);
    for (int j = 0; j < k + 1; ++j)
      for (int i = 0; i < k + 1; ++i) C1[j + ld * i] = M[j + ld * i];
    for (int j = 0; j < k + 2; ++j)
      for (int i = 0; i < k + 2; ++i) C2[j + ld * i] = M[j + ld * i];
    small_solve(C1, k + 1, ld, x1);
    small_solve(C2, k + 2, ld, x2);
    // P: Atemp = y + XX(0) dy + sum XX(i) dy_(n-i); E: derivative at t + dt
    adams_combine(c, c.ad_temp, xp.data(), k - 1);
    eom_from(c, c.ad_temp, c.ad_dnew);
    // C (order k+1) with int_par1 further EC iterations
    adams_combine(c, c.ad_temp, x1.data() + 1, k - 1);
    adams_axpy(c, c.ad_new, c.ad_temp, c.ad_dnew, x1[0]);
    for (int it = 0; it < c.int_par1; ++it) {
      eom_from(c, c.ad_new, c.ad_d1);
      adams_axpy(c, c.ad_new, c.ad_temp, c.ad_d1, x1[0]);
    }
    // C (order k+2)
    adams_combine(c, c.ad_temp, x2.data() + 1, k);
    adams_axpy(c, c.ad_new1, c.ad_temp, c.ad_dnew, x2[0]);
    for (int it = 0; it < c.int_par1; ++it) {
      eom_from(c, c.ad_new1, c.ad_d1);
      adams_axpy(c, c.ad_new1, c.ad_temp, c.ad_d1, x2[0]);
    }
    run_ovl(c, c.ad_plan);
    errmax = ovl_delta(c, c.ad_plan) / c.eps_int;
    check_status(c);
    if (!std::isfinite(errmax)) throw StatusError(MCTDH_ENONFINITE, "non-finite Adams error estimate");
    if (errmax < 1.0) break;
    dt = std::max(minscal * dt, safety * dt * pow(errmax, pow_shrink));
    if (dt < c.min_stepsize) throw StatusError(MCTDH_ESTEP, "The stepsize has become too small");
  }
  // errmax ** pow_shrink is +Infinity for errmax = 0 (IEEE), leaving maxscal * dt
  const double grow = (errmax > 0.0) ? pow(errmax, pow_shrink) : INFINITY;
  *hnext = std::min(std::min(maxscal * dt, dt * grow), c.writetime);
  *hdid = dt;
  // shift the history: dA_prev(:,1) = derivative at the old point (:366-373)
  cplx* oldest = c.ad_hist[k - 1];
  for (int i = k - 1; i > 0; --i) {
    c.ad_hist[i] = c.ad_hist[i - 1];
    c.ad_hprev[i] = c.ad_hprev[i - 1];
  }
  c.ad_hist[0] = c.ad_dcur;
  c.ad_hprev[0] = dt;
  c.ad_dcur = oldest;
  CK(cudaMemcpyAsync(c.d_y, c.ad_new1, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
  eom_from(c, c.d_y, c.ad_dcur);   // Calc_Derivs at tt + hdid
}

// One step of the Adams propagation on the resident state, bootstrapping with
// Cash-Karp for the first int_order steps (propagator.f90:156-198).  Returns
// whether the step was a bootstrap step.
bool adams_or_boot_step(Ctx& c, double t, double htry, double* hdid, double* hnext, long long* att) {
  adams_plan(c);
  const int k = c.int_order;
  if (!c.ad_valid) {
    eom_from(c, c.d_y, c.ad_dcur);   // propagator.f90:151
    c.ad_iprop = 0;
    c.ad_valid = true;
  }
  if (c.ad_iprop < k) {
    CK(cudaMemcpyAsync(c.ad_hist[k - 1 - c.ad_iprop], c.ad_dcur, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice,
                       c.st));
    CK(cudaMemcpyAsync(c.d_k[0], c.ad_dcur, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
    rkqs(c, t, htry, hdid, hnext, 1, att);
    eom_from(c, c.d_y, c.ad_dcur);
    c.ad_hprev[k - 1 - c.ad_iprop] = *hdid;
    c.ad_iprop++;
    return true;
  }
  adams_step(c, t, htry, hdid, hnext, att);
  return false;
}

// ---------------------------------------------------------------------------
// Bulirsch-Stoer (bsstep, mmid, pzextr, SetupBS; integrator.f90:384-608) on the
// resident state: modified midpoint sequences nSeq = 2, 4, .., 18, polynomial
// extrapolation to zero step, order window kOpt with the work model Ak.
// ---------------------------------------------------------------------------
const int BS_KMAXX = 8;
const int BS_NSEQ[9] = {2, 4, 6, 8, 10, 12, 14, 16, 18};
const double BS_SAFE1 = 0.25, BS_SAFE2 = 0.7, BS_REDMAX = 1e-5, BS_REDMIN = 0.7, BS_SCALMAX = 0.1;

void bs_plan(Ctx& c) {
  if (c.bs_planned) return;
  c.bs_Ak[1] = BS_NSEQ[0] + 1.0;
  for (int k = 1; k <= BS_KMAXX; ++k) c.bs_Ak[k + 1] = c.bs_Ak[k] + BS_NSEQ[k];
  for (int iq = 2; iq <= BS_KMAXX; ++iq)
    for (int k = 1; k < iq; ++k)
      c.bs_alf[k][iq] = pow(BS_SAFE1 * c.eps_int, (c.bs_Ak[k + 1] - c.bs_Ak[iq + 1]) /
                                                      ((c.bs_Ak[iq + 1] - c.bs_Ak[1] + 1.0) * (double)(2 * k + 1)));
  int kopt = BS_KMAXX;
  for (int ko = 2; ko < BS_KMAXX; ++ko)
    if (c.bs_Ak[ko + 1] > c.bs_Ak[ko] * c.bs_alf[ko - 1][ko]) {
      kopt = ko;
      break;
    }
  c.bs_kmax = kopt;
  c.bs_kopt = kopt;
  cplx** bufs[] = {&c.bs_save, &c.bs_d0, &c.bs_am, &c.bs_an, &c.bs_sw, &c.bs_d, &c.bs_seq, &c.bs_a0, &c.bs_a1};
  for (cplx** b : bufs) *b = c.ar.calloc_c(c.ntot);
  for (int q = 1; q <= BS_KMAXX + 1; ++q) c.bs_q[q] = c.ar.calloc_c(c.ntot);
  plan_ovl(c, c.bs_plan, c.bs_a0, c.bs_a1, (c.precision && c.eps_int >= 1e-5) ? 2 : 0);
  c.bs_planned = true;
}

// mmid: AOut (bs_seq) after nstep modified-midpoint steps of htot from bs_save
void bs_mmid(Ctx& c, double htot, int nstep) {
  const double dt = htot / nstep;
  StageArgs a;
  memset(&a, 0, sizeof(a));
  a.k[0] = c.bs_d0;
  a.c[0] = 1.0;
  a.nk = 1;
  CK(cudaMemcpyAsync(c.bs_am, c.bs_save, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
  launch_stage(c.bs_an, c.bs_save, a, dt, c.ntot, c.st);   // An = A0 + dt dA
  c.count();
  eom_from(c, c.bs_an, c.bs_d);
  cplx *am = c.bs_am, *an = c.bs_an, *sw = c.bs_sw;
  for (int n = 2; n <= nstep; ++n) {
    a.k[0] = c.bs_d;
    launch_stage(sw, am, a, 2.0 * dt, c.ntot, c.st);   // Aswap = Am + 2 dt D
    c.count();
    cplx* t = am;
    am = an;
    an = sw;
    sw = t;
    eom_from(c, an, c.bs_d);
  }
  launch_bs_final(c.bs_seq, am, an, c.bs_d, dt, c.ntot, c.st);
  c.count();
}

void bs_pzextr(Ctx& c, int iest, double test) {
  c.bs_tstore[iest] = test;
  BsExtr e;
  memset(&e, 0, sizeof(e));
  for (int q = 1; q <= BS_KMAXX + 1; ++q) e.q[q] = c.bs_q[q];
  e.iest = iest;
  for (int k1 = 1; k1 < iest; ++k1) {
    const double delta = 1.0 / (c.bs_tstore[iest - k1] - test);
    e.f1[k1] = test * delta;
    e.f2[k1] = c.bs_tstore[iest - k1] * delta;
  }
  launch_bs_extr(e, c.bs_seq, c.bs_a0, c.bs_a1, c.ntot, c.st);
  c.count();
}

// bsstep from d_y with its derivative in bs_d0; the accepted state lands in d_y.
void bsstep(Ctx& c, double t, double htry, double* hdid, double* hnext) {
  double dt = htry;
  CK(cudaMemcpyAsync(c.bs_save, c.d_y, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
  if (dt != c.bs_hnext || t != c.bs_tnew) {   // :428-431
    c.bs_first = true;
    c.bs_kopt = c.bs_kmax;
  }
  bool reduct = false, converged = false;
  double error[BS_KMAXX + 2] = {};
  const int kmax = c.bs_kmax;
  int k = 1;
  for (int guard = 0;; ++guard) {
    if (guard > 1000) throw StatusError(MCTDH_ESTEP, "Bulirsch-Stoer step not accepted");
    double red = BS_REDMIN;
    double errmax = 0.0;
    for (k = 1; k <= kmax; ++k) {
      c.bs_tnew = t + dt;
      bs_mmid(c, dt, BS_NSEQ[k - 1]);
      const double test = (dt / BS_NSEQ[k - 1]) * (dt / BS_NSEQ[k - 1]);
      bs_pzextr(c, k, test);
      if (k != 1) {
        run_ovl(c, c.bs_plan);
        errmax = ovl_delta(c, c.bs_plan) / c.eps_int;
        check_status(c);
        if (!std::isfinite(errmax)) throw StatusError(MCTDH_ENONFINITE, "non-finite Bulirsch-Stoer error estimate");
        error[k - 1] = pow(errmax / BS_SAFE1, 1.0 / (double)(2 * k - 1));
      }
      const int kopt = c.bs_kopt;
      if (k != 1 && (k >= kopt - 1 || c.bs_first)) {
        if (errmax < 1.0) {
          converged = true;
          break;
        }
        if (k == kmax || k == kopt + 1) {
          red = BS_SAFE2 / error[k - 1];
          break;
        } else if (k == kopt) {
          if (c.bs_alf[kopt - 1][kopt] < error[k - 1]) {
            red = 1.0 / error[k - 1];
            break;
          }
        } else if (kopt == kmax) {
          if (c.bs_alf[k - 1][kmax - 1] < error[k - 1]) {
            red = c.bs_alf[k - 1][kmax - 1] * BS_SAFE2 / error[k - 1];
            break;
          }
        } else if (c.bs_alf[k - 1][kopt] < error[k - 1]) {
          red = c.bs_alf[k - 1][kopt - 1] / error[k - 1];
          break;
        }
      }
    }
    if (converged) break;
    red = std::max(std::min(red, BS_REDMIN), BS_REDMAX);
    dt *= red;
    reduct = true;
  }
  *hdid = dt;
  c.bs_first = false;
  double workmin = 1e16, scal = 1.0;
  for (int kk = 1; kk <= k - 1; ++kk) {
    const double fact = std::max(error[kk], BS_SCALMAX);
    const double work = fact * c.bs_Ak[kk + 1];
    if (work < workmin) {
      scal = fact;
      workmin = work;
      c.bs_kopt = kk + 1;
    }
  }
  double hn = dt / scal;
  const int kopt = c.bs_kopt;
  if (kopt >= k && kopt != kmax && !reduct) {
    const double fact = std::max(scal / c.bs_alf[kopt - 1][kopt], BS_SCALMAX);
    if (c.bs_Ak[kopt + 1] * fact <= workmin) {
      hn = dt / fact;
      c.bs_kopt = kopt + 1;
    }
  }
  *hnext = hn;
  c.bs_hnext = hn;
  CK(cudaMemcpyAsync(c.d_y, c.bs_a0, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
}

// One Bulirsch-Stoer step of propagate_wf (propagator.f90:216-222): the
// derivative at the step start, then bsstep.
void bs_step(Ctx& c, double t, double htry, double* hdid, double* hnext) {
  bs_plan(c);
  eom_from(c, c.d_y, c.bs_d0);
  bsstep(c, t, htry, hdid, hnext);
}

// ---------------------------------------------------------------------------
// CMF2 (cmf2_base.f90:47-206) for DVR models
// ---------------------------------------------------------------------------
// H_B B (Calc_DHD_B) into out; input_ready: B is already in d_hbin (and d_hbin32),
// written there by the Lanczos normalisation that produced it.
void hb(Ctx& c, const cplx* B, cplx* out, bool with_dot = false, bool input_ready = false) {
  if (!input_ready) {
    if (B != c.d_hbin) CK(cudaMemcpyAsync(c.d_hbin, B, sizeof(cplx) * c.naconftot, cudaMemcpyDeviceToDevice, c.st));
    if (c.d_hbin32) {
      launch_to_f32(c.d_hbin32, c.d_hbin, c.naconftot, c.st);
      c.count();
    }
  }
  for (size_t i = 1; i < c.hb_chains.size(); ++i) run_prod(c, c.hb_chains[i]);
  launch_termsum(out, c.hbsum_d, c.nstates, c.hbsrc_d, c.naconftot, c.st, c.hb_prec,
                 with_dot ? c.hb_dot : FusedDot{nullptr, nullptr, nullptr, nullptr});
  c.count();
  c.hb_count++;
}

// <a|b> over the coefficient vector (FP64, deterministic); result left on the device
cplx* dot_dev(Ctx& c, const cplx* a, const cplx* b, long long n) {
  // plans are cached per context, keyed by the pointer pair
  auto key = std::make_pair((const void*)a, (const void*)b);
  DotPlan* P = c.dots.count(key) ? c.dots[key] : nullptr;
  if (!P) {
    P = new DotPlan();
    P->res = c.ar.calloc_c(1);
    P->partial = c.ar.calloc_c(DOT_BLOCKS);
    P->counter = (unsigned*)c.ar.alloc(sizeof(unsigned));
    CK(cudaMemset(P->counter, 0, sizeof(unsigned)));
    c.dots[key] = P;
  }
  {
    ProfScope ps(c, KP_HOLE, 8.0 * (double)n, 32.0 * (double)n);
    launch_dot(a, b, n, P->partial, P->counter, P->res, c.st);
    c.count();
  }
  return P->res;
}

cplx dot_now(Ctx& c, const cplx* a, const cplx* b, long long n) {
  cplx* d = dot_dev(c, a, b, n);
  cplx r;
  CK(cudaMemcpyAsync(&r, d, sizeof(cplx), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  return r;
}

const double EPS_B = 1e-8;  // cmf2_integration.f90:13
const int NKRYLOV_MAX = 20; // cmf2_integration.f90:11

// Lanczos (cmf2_integration.f90:30-103) as issue / check steps, so that the
// Krylov build can run on one stream while other work runs on another: lan_issue
// launches the next Krylov step (one CUDA graph) and the copy of its beta into
// pinned memory, lan_check applies the stopping rule once the stream is idle,
// lan_finish diagonalises the tridiagonal matrix and forms BT.  alpha_j, beta_j
// stay on the device (d_lan[0..19], d_lan[20..39]).
struct LanRun {
  const cplx* B0 = nullptr;
  double dt = 0.0, error = 0.0;
  int j = 0;          // 0 before the first step; then the index of the next Krylov vector
  int nk = 0;
  bool done = false;
};

void lan_issue(Ctx& c, LanRun& R) {
  RtScope rt(c, RT_LANCZOS, false);   // Lanczos (cmf2_integration.f90:30-103): the Krylov steps
  const long long n = c.naconftot;
  cplx* K = c.d_krylov;
  double* d_alpha = c.d_lan;
  double* d_beta = c.d_lan + NKRYLOV_MAX;
  double* h_beta = c.h_scal + 64;   // pinned
  if (R.j == 0) {
    // each Krylov step is a fixed launch sequence on fixed buffers: CUDA graphs
    const cplx* B0 = R.B0;
    run_graphed(c, 4, B0, [&] {
      // every normalisation also writes the next H_B input (d_hbin, d_hbin32)
      launch_lan_normalize(K, B0, dot_dev(c, B0, B0, n), nullptr, n, c.st, c.d_hbin, c.d_hbin32);
      c.count();
      // alpha = <K|H_B K> in the term sum, ||K'||^2 in the axpy
      hb(c, K, K + n, true, true);
      launch_lan_axpy(K + n, K, nullptr, c.hb_dot.res, nullptr, d_alpha, n, c.st, c.lan_nrm);
      launch_lan_normalize(K + n, K + n, c.lan_nrm.res, d_beta, n, c.st, c.d_hbin, c.d_hbin32);
      c.count(2);
    });
    CK(cudaMemcpyAsync(h_beta, d_beta, sizeof(double), cudaMemcpyDeviceToHost, c.st));
    return;
  }
  const int j = R.j;
  if (j == NKRYLOV_MAX) throw StatusError(MCTDH_EKRYLOV, "Maximum number of Krylov vectors reached");
  cplx* Kj = K + (long long)(j - 1) * n;
  cplx* Kn = K + (long long)j * n;
  cplx* Kp = K + (long long)(j - 2) * n;
  run_graphed(c, 3, Kn, [&] {
    hb(c, Kj, Kn, true, true);   // Kj is in d_hbin: the previous step's normalisation wrote it
    launch_lan_axpy(Kn, Kj, Kp, c.hb_dot.res, d_beta + (j - 2), d_alpha + (j - 1), n, c.st, c.lan_nrm);
    launch_lan_normalize(Kn, Kn, c.lan_nrm.res, d_beta + (j - 1), n, c.st, c.d_hbin, c.d_hbin32);
    c.count(2);
  });
  CK(cudaMemcpyAsync(h_beta + (j - 1), d_beta + (j - 1), sizeof(double), cudaMemcpyDeviceToHost, c.st));
}

// after the stream is idle: error = beta_1 |dt|, then error * beta_j / j * |dt| < eps_B
// (cmf2_integration.f90:64-80)
void lan_check(Ctx& c, LanRun& R) {
  const double* h_beta = c.h_scal + 64;
  if (R.j == 0) {
    R.error = h_beta[0] * fabs(R.dt);
    R.j = 2;
    return;
  }
  R.error = R.error * h_beta[R.j - 1] / (double)R.j * fabs(R.dt);
  if (R.error < EPS_B) {
    R.done = true;
    R.nk = R.j;
  } else {
    ++R.j;
  }
}

void lan_finish(Ctx& c, LanRun& R) {
  RtScope rt(c, RT_LANCZOS);   // one call per Lanczos run
  const int nk = R.nk;
  launch_jacobi_tridiag(c.d_lan, c.d_lan + NKRYLOV_MAX, nk, c.d_lan + 2 * NKRYLOV_MAX,
                        c.d_lan + 3 * NKRYLOV_MAX, c.d_status, c.st);
  c.count();
  c.lan_evals.assign(nk, 0.0);
  c.lan_evecs.assign(nk * nk, 0.0);
  CK(cudaMemcpyAsync(c.lan_evals.data(), c.d_lan + 2 * NKRYLOV_MAX, sizeof(double) * nk, cudaMemcpyDeviceToHost, c.st));
  CK(cudaMemcpyAsync(c.lan_evecs.data(), c.d_lan + 3 * NKRYLOV_MAX, sizeof(double) * nk * nk,
                     cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  check_status(c);
  c.lan_nk = nk;
}

// BT = sum_j BK_j * (sum_r U_jr U_1r exp(f alpha_r dt)), renormalised (:85-99)
void lan_combine(Ctx& c, cplx* BT, double dt) {
  RtScope rt(c, RT_LANCZOS, false);
  const long long n = c.naconftot;
  const int nk = c.lan_nk;
  std::vector<cplx> coef(nk, mkc(0, 0));
  for (int r = 0; r < nk; ++r) {
    double u1 = c.lan_evecs[0 + nk * r];
    cplx e = mkc(c.der.x * c.lan_evals[r] * dt, c.der.y * c.lan_evals[r] * dt);
    double mag = exp(e.x);
    cplx ex = mkc(mag * cos(e.y), mag * sin(e.y));
    for (int jj = 0; jj < nk; ++jj) {
      double ujr = c.lan_evecs[jj + nk * r];
      coef[jj] = cadd(coef[jj], cscale(ex, ujr * u1));
    }
  }
  CK(cudaMemcpyAsync(c.d_coef, coef.data(), sizeof(cplx) * nk, cudaMemcpyHostToDevice, c.st));
  launch_gemv_cols(BT, c.d_krylov, n, c.d_coef, nk, n, c.st);
  launch_lan_normalize(BT, BT, dot_dev(c, BT, BT, n), nullptr, n, c.st);
  c.count(2);
}

// Lanczos from B0 (device, naconftot) into BT on the context's stream; build =
// false reuses the last Krylov space (cmf2_base.f90:189).
void lanczos(Ctx& c, const cplx* B0, cplx* BT, double dt, bool build) {
  if (build) {
    LanRun R;
    R.B0 = B0;
    R.dt = dt;
    while (!R.done) {
      lan_issue(c, R);
      CK(cudaStreamSynchronize(c.st));
      lan_check(c, R);
    }
    lan_finish(c, R);
  }
  lan_combine(c, BT, dt);
}

// operators and mean fields on the state y (Calc_rho1mode, Calc_h1mode,
// Calc_MeanField, Calc_rhom1MF): one EOM into d_out (the derivative is unused).
void operators_and_mf(Ctx& c, const cplx* y, bool reginv = true) {
  run_graphed(c, reginv ? 2 : 5, y, [&] {
    if (y != c.d_in) CK(cudaMemcpyAsync(c.d_in, y, sizeof(cplx) * c.ntot, cudaMemcpyDeviceToDevice, c.st));
    eom(c, c.d_out, true, reginv);
  });
}

void copy_dev(Ctx& c, cplx* dst, const cplx* src, long long n) {
  CK(cudaMemcpyAsync(dst, src, sizeof(cplx) * n, cudaMemcpyDeviceToDevice, c.st));
}

// h1mode only (no mean fields) on the SPFs of y: used before the back-propagation.
void h1_only(Ctx& c, const cplx* y) {
  RtScope rt(c, RT_H1MODE);
  copy_dev(c, c.d_in + c.naconftot, y + c.naconftot, c.dimpsi);
  if (!c.modes_gwp.empty()) {
    // Calc_S00 and Calc_h1mode of the Gaussian modes (cmf2_base.f90:158-163)
    launch_gwp_ovl(c.gs_d, (int)c.gs_h.size(), c.st);
    launch_gwp_h1(c.gh1_d, (int)c.gh1_h.size(), c.st);
    c.count(2);
  }
  launch_h1(c.h1_d, (int)c.h1_h.size(), c.h1_maxn2, c.h1_smem, true, c.st, c.precision);
  launch_matsum(c.msum_d, (int)c.msum_h.size(), c.msum_src_d, c.st);
  c.count(3);
}

// SPF integration of all DVR modes with frozen mean fields, in lockstep: one
// launch per Runge-Kutta stage covers every mode, each mode keeps the step
// control of propagate_SPF / rk_SPF_ck (cmf2_base.f90:210-260,
// cmf2_integration.f90:105-253) with its own step length.  Modes are
// independent (their SPF equations see only their own SPFs and the frozen mean
// fields), so the result equals mode-by-mode integration.
struct CmfState {
  bool planned = false;
  cplx *B0, *BHalf, *B02, *psiHalf, *psiHalf2, *AHalf;  // full-length vectors (ntot)
  cplx* ytmp;
  std::vector<H1Desc> h1;       // operators on the current SPFs (h1mode frozen)
  H1Desc* h1_d = nullptr;
  unsigned char* elem_mode = nullptr;   // mode of every psi element
  double* dt_mode = nullptr;            // device, per mode
  int* accept = nullptr;                // device, per mode
  double* err_mode = nullptr;           // device, per mode
  HoleBatch err_holes;                  // (dphi)^H dphi per (mode, state block)
  RedBatch err_red;
  std::vector<SpfErrDesc> errd_h;
  SpfErrDesc* errd_d = nullptr;
  long long rk_iters = 0;
  // the step-start operators (h1mode, h·phi, the pre-summed single-mode
  // operators, rho, the mean fields) of grid-mode models, saved after their
  // evaluation so that a rejected attempt's retry from the same state restores
  // them instead of evaluating them again
  std::vector<SnapSeg> opseg_h;
  SnapSeg* opseg_d = nullptr;
  long long opE = 0;
  cplx* opsave = nullptr;
  // the Krylov space of the step-start Lanczos run (its vectors, alpha and beta):
  // a retry from the same state with a shorter step uses its leading vectors
  cplx* krylov0 = nullptr;
  double* lan0 = nullptr;
  std::vector<double> beta0;
  bool k0_valid = false;
  // Gaussian modes (cmf2_base.f90): the D matrices of every (mode, set) block,
  // concatenated into one vector per role; B = D^H S A is the propagated vector
  bool gwp = false;
  long long nD = 0;
  cplx *DD0 = nullptr, *DDHalf = nullptr, *DDHalf2 = nullptr;   // DD0, DDHalf, DDHalf2 of cmf2
  cplx *Din = nullptr, *Dtmp = nullptr, *DhS = nullptr;         // stage input, 5th-order result, D^H S
  cplx* Dk[7] = {};                                             // stage derivatives dDD
  unsigned char* d_elem_mode = nullptr;                         // mode of every D element
  std::vector<GwpIsqrtDesc> isq_h;
  GwpIsqrtDesc* isq_d = nullptr;
  std::vector<GwpDhdDesc> dhd0_h, dhd2_h;                       // D^H h D with DD0 / DDHalf2
  GwpDhdDesc *dhd0_d = nullptr, *dhd2_d = nullptr;
  std::vector<GwpDDerivDesc> dder_h;
  GwpDDerivDesc* dder_d = nullptr;
  std::vector<GwpOvlDesc> gerr_h;                               // Calc_Err_SPF overlaps
  GwpOvlDesc* gerr_d = nullptr;
  std::vector<ProdBatch> a2b, b2a_half, b2a_end;                // A_to_B, B_to_A chains
  double* h_dt = nullptr;    // pinned host copies: per-mode step lengths, errors, accept flags
  double* h_err = nullptr;
  int* h_acc = nullptr;
  ~CmfState() {
    if (h_dt) cudaFreeHost(h_dt);
    if (h_err) cudaFreeHost(h_err);
    if (h_acc) cudaFreeHost(h_acc);
  }
};
std::map<const Ctx*, CmfState*> g_cmf;

void stage_modes(Ctx& c, CmfState& S, cplx* out, const cplx* base, const double* coef, int nk) {
  StageArgs a;
  memset(&a, 0, sizeof(a));
  int n = 0;
  for (int j = 0; j < nk; ++j) {
    if (coef[j] == 0.0) continue;
    a.k[n] = c.d_k[j];
    a.c[n] = coef[j];
    ++n;
  }
  a.nk = n;
  ProfScope ps(c, KP_ELEM);
  launch_stage_modes(out, base, a, S.dt_mode, S.elem_mode, c.naconftot, c.dimpsi, c.st);
  c.count();
}

// the same combination on the D vectors of the Gaussian modes (rk_SPF_ck DDtemp)
void stage_D(Ctx& c, CmfState& S, cplx* out, const cplx* base, const double* coef, int nk) {
  if (!S.gwp) return;
  StageArgs a;
  memset(&a, 0, sizeof(a));
  int n = 0;
  for (int j = 0; j < nk; ++j) {
    if (coef[j] == 0.0) continue;
    a.k[n] = S.Dk[j];
    a.c[n] = coef[j];
    ++n;
  }
  a.nk = n;
  ProfScope ps(c, KP_ELEM);
  launch_stage_modes(out, base, a, S.dt_mode, S.d_elem_mode, 0, S.nD, c.st);
  c.count();
}

// Calc_Der_SPF (cmf2_derivatives.f90:84-235) of every mode on the SPFs in d_in
// (and the D matrices in S.Din) with frozen mean fields: grid modes through the
// h1 and SPF-tile kernels; Gaussian modes through S00, its Tikhonov inverse,
// h1mode, C and Y with the frozen density matrices and mean fields, the
// Tikhonov solve (der_factor * x into out) and dD = -tau D into Dout.
void spf_eval_all(Ctx& c, CmfState& S, cplx* out, cplx* Dout) {
  if (!c.modes_dvr.empty()) {
    RtScope rt(c, RT_SPF_DVR);   // Calc_Der_SPF (cmf2_derivatives.f90:84-235), h1 refresh included
    {
      ProfScope ps(c, KP_H1);
      launch_h1(S.h1_d, (int)S.h1.size(), c.h1_maxn2, c.h1_smem, false, c.st, c.precision);
    }
    {
      ProfScope ps(c, KP_SPF);
      launch_spf(c.spf_d, (int)c.spf_h.size(), c.spf_tiles, c.spfop_d, out, c.der, c.d_status, c.st, c.precision, c.spf_nf);
    }
    c.count(4);
  }
  if (S.gwp) {
    RtScope rt(c, RT_SPF_GWP);
    gwp_setup_run(c);
    gwp_solve_run(c, out);
    ProfScope ps(c, KP_GWP);
    launch_gwp_dderiv(S.dder_d, (int)S.dder_h.size(), S.Din, Dout, c.st);
    c.count();
  }
}

// Per state, mode products over the Gaussian modes with mat(i, set), src -> dst:
// one batch per Gaussian mode (A_to_B / B_to_A, cmf2_base.f90:264-345).
template <typename F>
void plan_gwp_chain(Ctx& c, std::vector<ProdBatch>& B, const cplx* src, cplx* dst, F mat) {
  const int ng = (int)c.modes_gwp.size();
  B.assign(ng, ProdBatch());
  for (int s = 0; s < c.nstates; ++s) {
    std::vector<int> sh = c.shape_of(s);
    const cplx* cur = src + c.aoff[s];
    for (int i = 0; i < ng; ++i) {
      const int m = c.modes_gwp[i];
      cplx* out = (i + 1 == ng) ? dst + c.aoff[s] : c.ar.calloc_c(c.naconf[s]);
      B[i].add(cur, out, mat(i, set_of(c, m, s)), sh[m], 0, sh, m, sh[m], mkc(1, 0), 0);
      cur = out;
    }
  }
  for (auto& b : B) b.finalize(c.ar);
}

// CMF2 buffers and plans of the Gaussian modes: D vectors, S^-1/2 by Cholesky,
// D^H h D, dD = -tau D, the SPF error overlaps, A_to_B and B_to_A.
void plan_cmf_gwp(Ctx& c, CmfState& S, std::vector<unsigned char>& em) {
  const int f = c.nmodes;
  const int ng = (int)c.modes_gwp.size();
  S.gwp = true;
  std::vector<std::vector<long long>> doff(ng, std::vector<long long>(c.nstates, 0));
  std::vector<unsigned char> dem;
  for (int i = 0; i < ng; ++i) {
    const int m = c.modes_gwp[i];
    const int nsets = c.multiset[m] ? c.nstates : 1;
    for (int s = 0; s < nsets; ++s) {
      const int n = c.m_of(m, s);
      doff[i][s] = S.nD;
      S.nD += (long long)n * n;
      dem.insert(dem.end(), (size_t)n * n, (unsigned char)m);
      const long long o = c.ipsi[m + f * s], len = (long long)c.nmodedof[m] * n;
      for (long long q = 0; q < len; ++q) em[o + q] = (unsigned char)m;
    }
  }
  S.DD0 = c.ar.calloc_c(S.nD);
  S.DDHalf = c.ar.calloc_c(S.nD);
  S.DDHalf2 = c.ar.calloc_c(S.nD);
  S.Din = c.ar.calloc_c(S.nD);
  S.Dtmp = c.ar.calloc_c(S.nD);
  S.DhS = c.ar.calloc_c(S.nD);
  for (int j = 0; j < 7; ++j) S.Dk[j] = c.ar.calloc_c(S.nD);
  S.d_elem_mode = upload_vec(c.ar, dem);
  for (int i = 0; i < ng; ++i) {
    const int m = c.modes_gwp[i];
    const double* a = c.gwpa_d + (size_t)c.gwp_lda * c.ns00max * i;
    const int nsets = c.multiset[m] ? c.nstates : 1;
    for (int s = 0; s < nsets; ++s) {
      const int n = c.m_of(m, s);
      GwpIsqrtDesc q;
      memset(&q, 0, sizeof(q));
      q.S = c.s00[i][s][s];
      q.D = S.DD0 + doff[i][s];
      q.DhS = S.DhS + doff[i][s];
      q.n = n;
      S.isq_h.push_back(q);
      GwpDDerivDesc dd;
      memset(&dd, 0, sizeof(dd));
      dd.tau = c.tau[i][s];
      dd.off = doff[i][s];
      dd.n = n;
      S.dder_h.push_back(dd);
      cplx* mat = c.ar.calloc_c((long long)n * n);
      GwpOvlDesc g;
      memset(&g, 0, sizeof(g));
      g.xi1 = psi_block(c, c.d_tmp, m, s);
      g.xi2 = psi_block(c, c.d_err, m, s);
      g.a = a;
      g.out = mat;
      g.nmd = c.nmodedof[m];
      g.lda = c.gwp_lda;
      g.n1 = n;
      g.n2 = n;
      g.kind = 3;
      S.gerr_h.push_back(g);
      SpfErrDesc ed;
      ed.ds = mat;
      ed.rho = c.multiset[m] ? c.rho[m][s] : c.rho_ave[m];
      ed.n = n;
      ed.mode = m;
      S.errd_h.push_back(ed);
    }
    for (int k = 0; k < c.noper[m]; ++k) {
      if (c.is_identity[m + f * k] || !c.ham_op[m][k]) continue;
      const int l = c.oper[m][k][0], r = c.oper[m][k][1];
      GwpDhdDesc d;
      memset(&d, 0, sizeof(d));
      d.h = c.hmat[m][k];
      d.out = c.dhd[i][k];
      d.n1 = c.m_of(m, l);
      d.n2 = c.m_of(m, r);
      d.same_state = (l == r);
      d.D1 = S.DD0 + doff[i][set_of(c, m, l)];
      d.D2 = S.DD0 + doff[i][set_of(c, m, r)];
      S.dhd0_h.push_back(d);
      d.D1 = S.DDHalf2 + doff[i][set_of(c, m, l)];
      d.D2 = S.DDHalf2 + doff[i][set_of(c, m, r)];
      S.dhd2_h.push_back(d);
    }
  }
  S.isq_d = upload_vec(c.ar, S.isq_h);
  S.dder_d = upload_vec(c.ar, S.dder_h);
  S.gerr_d = upload_vec(c.ar, S.gerr_h);
  S.dhd0_d = upload_vec(c.ar, S.dhd0_h);
  S.dhd2_d = upload_vec(c.ar, S.dhd2_h);
  plan_gwp_chain(c, S.a2b, c.d_y, S.B0, [&](int i, int s) { return (const cplx*)(S.DhS + doff[i][s]); });
  plan_gwp_chain(c, S.b2a_half, S.BHalf, S.AHalf, [&](int i, int s) { return (const cplx*)(S.DDHalf + doff[i][s]); });
  plan_gwp_chain(c, S.b2a_end, S.B02, c.d_y, [&](int i, int s) { return (const cplx*)(S.DDHalf2 + doff[i][s]); });
}

void plan_cmf(Ctx& c, CmfState& S) {
  const int f = c.nmodes;
  S.B0 = c.ar.calloc_c(c.ntot);
  S.BHalf = c.ar.calloc_c(c.ntot);
  S.B02 = c.ar.calloc_c(c.ntot);
  S.psiHalf = c.ar.calloc_c(c.ntot);
  S.psiHalf2 = c.ar.calloc_c(c.ntot);
  S.AHalf = c.ar.calloc_c(c.ntot);
  S.ytmp = c.ar.calloc_c(c.ntot);
  for (auto hd : c.h1_h) {
    hd.h = nullptr;   // mean fields and h1mode stay frozen; only ophi is refreshed
    S.h1.push_back(hd);
  }
  S.h1_d = upload_vec(c.ar, S.h1);
  std::vector<unsigned char> em((size_t)std::max<long long>(c.dimpsi, 1), 0);
  std::vector<HoleRef> hrefs;
  for (int m : c.modes_dvr) {
    for (int s = 0; s < c.nstates; ++s) {
      if (!c.multiset[m] && s > 0) break;
      const int n = c.m_of(m, s);
      const long long o = c.ipsi[m + f * s], len = (long long)c.gmode[m] * n;
      for (long long i = 0; i < len; ++i) em[o + i] = (unsigned char)m;
      cplx* mat = c.ar.calloc_c((long long)n * n);
      cplx* p = S.ytmp + c.naconftot + o;
      int h = S.err_holes.add(c.ar, p, p, c.gmode[m], 1, n, n);
      hrefs.push_back(HoleRef{h, S.err_red.add_target(mat, n, n, n, 1), mkc(1, 0)});
      SpfErrDesc ed;
      ed.ds = mat;
      ed.rho = c.multiset[m] ? c.rho[m][s] : c.rho_ave[m];
      ed.n = n;
      ed.mode = m;
      S.errd_h.push_back(ed);
    }
  }
  if (!c.modes_gwp.empty()) plan_cmf_gwp(c, S, em);
  if (c.modes_gwp.empty()) {
    long long off = 0;
    auto seg = [&](cplx* p, long long n) {
      if (!p || n <= 0) return;
      S.opseg_h.push_back(SnapSeg{p, off, 0, 0});
      off += n;
    };
    for (int m : c.modes_dvr) {
      for (int k = 0; k < c.noper[m]; ++k) {
        const long long n1 = c.m_of(m, c.oper[m][k][0]), n2 = c.m_of(m, c.oper[m][k][1]);
        if (!c.is_identity[m + f * k]) seg(c.hmat[m][k], n1 * n2);
        seg(c.ophi[m][k], (long long)c.gmode[m] * n2);
        seg(c.mf[m][k], n1 * n2);
      }
      for (int st = 0; st < c.nstates; ++st)
        if (c.rho[m][st]) seg(c.rho[m][st], (long long)c.m_of(m, st) * c.m_of(m, st));
      if (c.rho_ave[m]) seg(c.rho_ave[m], (long long)c.m_of(m, 0) * c.m_of(m, 0));
    }
    for (const MatSumDesc& md : c.msum_h) seg(md.out, (long long)md.n1 * md.n2);
    S.opE = off;
    if (off > 0) {
      S.opseg_d = upload_vec(c.ar, S.opseg_h);
      S.opsave = c.ar.calloc_c(off);
    }
    S.krylov0 = c.ar.calloc_c(c.naconftot * (NKRYLOV_MAX + 1));
    S.lan0 = (double*)c.ar.alloc(sizeof(double) * (3 * NKRYLOV_MAX + NKRYLOV_MAX * NKRYLOV_MAX));
  }
  S.elem_mode = upload_vec(c.ar, em);
  // the SPF error norms: compensated split FP32 (~1e-13) in the split modes
  S.err_holes.prec = c.precision ? 2 : 0;
  S.err_holes.finalize(c.ar);
  for (auto& hr : hrefs) S.err_red.add_term(hr.target, S.err_holes.h[hr.hole], hr.alpha);
  S.err_red.finalize(c.ar);
  if (S.errd_h.size() > 256) throw StatusError(MCTDH_EUNSUPPORTED, "more than 256 (mode, state) SPF blocks");
  S.errd_d = upload_vec(c.ar, S.errd_h);
  S.dt_mode = (double*)c.ar.alloc(sizeof(double) * 64);
  S.accept = (int*)c.ar.alloc(sizeof(int) * 64);
  S.err_mode = (double*)c.ar.alloc(sizeof(double) * 64);
  CK(cudaMallocHost(&S.h_dt, sizeof(double) * 64));
  CK(cudaMallocHost(&S.h_err, sizeof(double) * 64));
  CK(cudaMallocHost(&S.h_acc, sizeof(int) * 64));
  if (f > 64) throw StatusError(MCTDH_EUNSUPPORTED, "more than 64 modes");
  S.planned = true;
}

// The SPF integration of one CMF2 half step as issue / check steps (like LanRun),
// so it can run on a second stream while the Lanczos build runs on the first.
struct SpfRun {
  double dt_total = 0.0;
  cplx* y = nullptr;
  cplx* Dy = nullptr;
  bool dp = false, finished = false;
  int iter = 0;
  std::vector<double> done, dtry;
  std::vector<int> active;
};

void spf_begin(Ctx& c, SpfRun& R, double dt_total, cplx* y, cplx* Dy) {
  if (c.int_type_psi != 1 && c.int_type_psi != 2)
    throw StatusError(MCTDH_EUNSUPPORTED, "SPF integrator must be rk45 (1) or dopri (2)");
  const int f = c.nmodes;
  R.dt_total = dt_total;
  R.y = y;
  R.Dy = Dy;
  R.dp = c.int_type_psi == 2;
  R.done.assign(f, 0.0);
  R.dtry.assign(f, 0.0);
  R.active.assign(f, 0);
  for (int m : c.modes_dvr) {
    R.active[m] = 1;
    R.dtry[m] = dt_total;
  }
  for (int m : c.modes_gwp) {
    R.active[m] = 1;
    R.dtry[m] = dt_total;
  }
  R.finished = false;
  for (int m = 0; m < f; ++m) R.finished = R.finished || R.active[m];
  R.finished = !R.finished;
}

// one RK attempt of every active mode on the context's stream, and the copy of
// the per-mode errors into pinned memory
void spf_issue(Ctx& c, CmfState& S, SpfRun& R) {
  const int f = c.nmodes;
  const bool dp = R.dp;
  cplx* y = R.y;
  cplx* Dy = R.Dy;
  const long long nA = c.naconftot;
  if (R.iter > 100000) throw StatusError(MCTDH_ESTEP, "SPF integration did not finish");
  ++R.iter;
  ++S.rk_iters;
  for (int m = 0; m < 64; ++m) S.h_dt[m] = (m < f && R.active[m]) ? R.dtry[m] : 0.0;
  CK(cudaMemcpyAsync(S.dt_mode, S.h_dt, sizeof(double) * 64, cudaMemcpyHostToDevice, c.st));
  // one RK attempt of every mode: the same launches on the same buffers each
  // iteration (the step lengths live in S.dt_mode), so it runs as a CUDA graph
  run_graphed(c, 1, y, [&] {
    copy_dev(c, c.d_in + nA, y + nA, c.dimpsi);
    if (S.gwp) copy_dev(c, S.Din, Dy, S.nD);
    spf_eval_all(c, S, c.d_k[0], S.Dk[0]);
    for (int st = 1; st < 6; ++st) {
      stage_modes(c, S, c.d_in, y, dp ? DP_B[st] : CK_B[st], st);
      stage_D(c, S, S.Din, Dy, dp ? DP_B[st] : CK_B[st], st);
      spf_eval_all(c, S, c.d_k[st], S.Dk[st]);
    }
    if (dp) {
      // the 7th stage is the derivative at the 5th-order solution (:386-393)
      stage_modes(c, S, c.d_in, y, DP_C, 6);
      stage_D(c, S, S.Din, Dy, DP_C, 6);
      spf_eval_all(c, S, c.d_k[6], S.Dk[6]);
      stage_modes(c, S, c.d_tmp, y, DP_C, 6);
      stage_D(c, S, S.Dtmp, Dy, DP_C, 6);
      stage_modes(c, S, c.d_err, y, DP_D, 7);
    } else {
      stage_modes(c, S, c.d_tmp, y, CK_C, 6);
      stage_D(c, S, S.Dtmp, Dy, CK_C, 6);
      stage_modes(c, S, c.d_err, y, CK_D, 6);
    }
    StageArgs a;
    memset(&a, 0, sizeof(a));
    a.k[0] = c.d_err + nA;
    a.c[0] = -1.0;
    a.nk = 1;
    launch_stage(S.ytmp + nA, c.d_tmp + nA, a, 1.0, c.dimpsi, c.st);
    c.count();
    run_hole(c, S.err_holes);
    run_red(c, S.err_red);
    if (S.gwp) {
      launch_gwp_ovl(S.gerr_d, (int)S.gerr_h.size(), c.st);
      c.count();
    }
    launch_spf_err(S.errd_d, (int)S.errd_h.size(), S.err_mode, f, c.st);
    c.count();
  });
  CK(cudaMemcpyAsync(S.h_err, S.err_mode, sizeof(double) * f, cudaMemcpyDeviceToHost, c.st));
}

// after the stream is idle: each mode's rk_SPF_ck / propagate_SPF control
// (cmf2_integration.f90:231-248, cmf2_base.f90:225-237), then the accepted modes'
// SPFs (and D matrices) copied into y on the context's stream
void spf_check(Ctx& c, CmfState& S, SpfRun& R) {
  const int f = c.nmodes;
  const double errcon = pow(5.0 / RK_SAFETY, 1.0 / RK_PGROW);
  for (int m = 0; m < 64; ++m) S.h_acc[m] = 0;
  for (int m = 0; m < f; ++m) {
    if (!R.active[m]) continue;
    const double error = S.h_err[m] / c.eps_psi;
    if (!std::isfinite(error)) throw StatusError(MCTDH_ENONFINITE, "non-finite SPF error estimate");
    if (error >= 1.0) {   // retry with a shorter step (rk_SPF_ck :231)
      R.dtry[m] = std::max(RK_MINSCAL * R.dtry[m], RK_SAFETY * R.dtry[m] * pow(error, RK_PSHRNK));
      continue;
    }
    S.h_acc[m] = 1;
    const double hdid = R.dtry[m];
    double hnext = (error > errcon) ? RK_SAFETY * hdid * pow(error, RK_PGROW) : hdid * RK_MAXSCAL;
    R.done[m] += hdid;
    if (R.done[m] >= R.dt_total) {   // propagate_SPF :229
      R.active[m] = 0;
      continue;
    }
    hnext = std::max(hnext, c.min_stepsize * 2);
    double step = (R.dt_total - R.done[m]) / ((double)(long long)((R.dt_total - R.done[m]) / hnext) + 1);
    R.dtry[m] = std::min(step, R.dt_total - R.done[m]);
  }
  CK(cudaMemcpyAsync(S.accept, S.h_acc, sizeof(int) * 64, cudaMemcpyHostToDevice, c.st));
  launch_masked_copy(R.y, c.d_tmp, S.elem_mode, S.accept, c.naconftot, c.dimpsi, c.st);
  c.count();
  if (S.gwp) {
    launch_masked_copy(R.Dy, S.Dtmp, S.d_elem_mode, S.accept, 0, S.nD, c.st);
    c.count();
  }
  bool any = false;
  for (int m = 0; m < f; ++m) any = any || R.active[m];
  R.finished = !any;
}

// propagate_SPF for every mode over dt_total, on the psi part of y and, for
// Gaussian modes, the D matrices in Dy (cmf2_base.f90:210-260): Cash-Karp
// (rk_SPF_ck, cmf2_integration.f90:105-253) for int_type_psi 1, Dormand-Prince
// (rk_SPF_dp, :257-412) for 2.
void propagate_spf_all(Ctx& c, CmfState& S, double dt_total, cplx* y, cplx* Dy) {
  SpfRun R;
  spf_begin(c, R, dt_total, y, Dy);
  while (!R.finished) {
    spf_issue(c, S, R);
    CK(cudaStreamSynchronize(c.st));
    spf_check(c, S, R);
  }
  if (S.gwp) check_status(c);
}

CmfState& cmf_state(Ctx& c) {
  if (c.member) throw StatusError(MCTDH_EUNSUPPORTED, "ensemble members integrate with RK");
  CmfState*& Sp = g_cmf[&c];
  if (!Sp) {
    Sp = new CmfState();
    plan_cmf(c, *Sp);
  }
  return *Sp;
}

// One CMF2 attempt of length hdid from d_y (cmf2_base.f90:76-176); returns
// max(err_A, err_psi) / eps_int and leaves BHalf / psiHalf2 for cmf2_accept.
// ---------------------------------------------------------------------------
// Learned mean-field extrapolation inside CMF2.  A snapshot is every density
// matrix and mean field of the grid modes (the inputs of Calc_rhom1MF).  The
// history holds the snapshots computed at the half steps of the last accepted
// CMF2 steps.  With a trained network attached and a full history, the mean
// fields at a step start (the first evaluation of cmf2_base.f90:78-87) come from
// the polynomial extrapolation of that history plus the network's residual
// instead of the chains and contractions of an EOM evaluation; h1mode (all the
// A-vector propagation uses) and the density matrices (one contraction of A per
// mode and state) are still computed, so rho^-1 sees no prediction error.  The half-step
// mean fields (:122-130) are always computed; the extrapolation's prediction for
// the half step is checked against them, and a step whose mismatch exceeds the
// tolerance is redone with the plain scheme.  One mean-field evaluation per
// step instead of two.
// ---------------------------------------------------------------------------
struct MfxState {
  long long E = 0;
  std::vector<SnapSeg> segs_h;
  SnapSeg* segs_d = nullptr;
  cplx* hist[MFX_NHIST] = {};
  double thist[MFX_NHIST] = {};
  int nhist = 0, head = 0;         // head: index of the newest entry
  double* S = nullptr;             // device: feature scale of the current prediction
  // half: the half-step snapshot of the current attempt; start: the step-start
  // snapshot (recorded steps); pred0 / pred1: the predictions at the step start
  // and at the half step
  cplx *half = nullptr, *start = nullptr, *pred0 = nullptr, *pred1 = nullptr, *now = nullptr, *backup = nullptr;
  mctdh_mlp* mlp = nullptr;
  double fscale[MFX_NFEAT] = {}, tscale[MFX_NOUT] = {}, tol = 0.0;
  int order[2] = {MFX_NHIST - 1, MFX_NHIST - 1};   // polynomial order at the step start / half step
  bool recording = false;
  std::vector<double> rec_t0, rec_h;
  std::vector<cplx> rec_s0, rec_sh;
  long long mlp_steps = 0, fallbacks = 0, rejected = 0;
  double last_rel = -1.0;          // relative step-end mismatch of the last validated prediction
  double gate = 1e300;             // extrapolate only after a step whose first attempt had error < gate
  double last_first_err = 0.0;     // error / eps_int of the first attempt of the last step
  std::vector<double> log;         // per CMF2 attempt: t, h, error, extrapolated (0/1), step-end mismatch
  HoleBatch dh;                     // ||now - pred1||^2 and ||now||^2
  RedBatch dr;
  cplx* dres = nullptr;
  cplx* diff = nullptr;
};
std::map<const Ctx*, MfxState*> g_mfx;

MfxState& mfx_state(Ctx& c) {
  MfxState*& M = g_mfx[&c];
  if (M) return *M;
  M = new MfxState();
  long long off = 0;
  const int f = c.nmodes;
  for (int m : c.modes_dvr) {
    for (int s = 0; s < c.nstates; ++s) {
      M->segs_h.push_back(SnapSeg{c.rho[m][s], off, 1, 0});
      off += (long long)c.m_of(m, s) * c.m_of(m, s);
    }
    if (!c.multiset[m]) {
      M->segs_h.push_back(SnapSeg{c.rho_ave[m], off, 1, 0});
      off += (long long)c.m_of(m, 0) * c.m_of(m, 0);
    }
    for (int k = 0; k < c.noper[m]; ++k) {
      if (c.is_identity[m + f * k] || !c.ham_op[m][k]) continue;
      M->segs_h.push_back(SnapSeg{c.mf[m][k], off, 0, 0});
      off += (long long)c.m_of(m, c.oper[m][k][0]) * c.m_of(m, c.oper[m][k][1]);
    }
  }
  M->E = off;
  M->segs_d = upload_vec(c.ar, M->segs_h);
  for (auto& h : M->hist) h = c.ar.calloc_c(off);
  M->half = c.ar.calloc_c(off);
  M->start = c.ar.calloc_c(off);
  M->pred0 = c.ar.calloc_c(off);
  M->pred1 = c.ar.calloc_c(off);
  M->now = c.ar.calloc_c(off);
  M->diff = c.ar.calloc_c(off);
  M->backup = c.ar.calloc_c(c.ntot);
  M->dres = c.ar.calloc_c(2);
  M->S = (double*)c.ar.alloc(sizeof(double) * 2);
  int h1 = M->dh.add(c.ar, M->diff, M->diff, off, 1, 1, 1);
  int h2 = M->dh.add(c.ar, M->now, M->now, off, 1, 1, 1);
  M->dh.finalize(c.ar);
  M->dr.add_term(M->dr.add_target(M->dres, 1, 1, 1, 0), M->dh.h[h1], mkc(1, 0));
  M->dr.add_term(M->dr.add_target(M->dres + 1, 1, 1, 1, 0), M->dh.h[h2], mkc(1, 0));
  M->dr.finalize(c.ar);
  return *M;
}

void snap_gather(Ctx& c, MfxState& M, cplx* flat) {
  launch_snap(M.segs_d, (int)M.segs_h.size(), flat, M.E, 0, c.st);
  c.count();
}

// relative distance of the computed half-step snapshot (M.now) from its prediction
double snap_rel_diff(Ctx& c, MfxState& M) {
  StageArgs a;
  memset(&a, 0, sizeof(a));
  a.k[0] = M.pred1;
  a.c[0] = -1.0;
  a.nk = 1;
  launch_stage(M.diff, M.now, a, 1.0, M.E, c.st);
  run_hole(c, M.dh);
  run_red(c, M.dr);
  cplx r[2];
  CK(cudaMemcpyAsync(r, M.dres, sizeof(cplx) * 2, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  return sqrt(r[0].x / std::max(r[1].x, 1e-300));
}

// Lagrange weights at tau of the polynomial through the points ts[first..n-1]
// (zero weight for the earlier points).
static void lagrange_tail(const double* ts, int n, int first, double tau, double* w) {
  for (int j = 0; j < n; ++j) {
    w[j] = 0.0;
    if (j < first) continue;
    double p = 1.0;
    for (int k = first; k < n; ++k)
      if (k != j) p *= (tau - ts[k]) / (ts[j] - ts[k]);
    w[j] = p;
  }
}

// Predict the snapshots at the times tau0 (a step start) and tau1 (its half step)
// from the history: quartic extrapolation through the last five half-step
// snapshots plus the network's residual, whose inputs are the Newton increments
// of orders 1-4 (mfx_features_kernel).  Results in M.pred0 and M.pred1.
void mfx_predict(Ctx& c, MfxState& M, double tau0, double tau1) {
  const int NH = MFX_NHIST;
  MfxHist hz;
  double ts[MFX_NHIST];
  for (int j = 0; j < NH; ++j) {
    const int idx = (M.head + 1 + j) % NH;   // oldest first
    hz.z[j] = M.hist[idx];
    ts[j] = M.thist[idx];
  }
  MfxCoef cf;
  memset(&cf, 0, sizeof(cf));
  const double taus[2] = {tau0, tau1};
  for (int tau = 0; tau < 2; ++tau) {
    double prev[MFX_NHIST] = {};
    prev[NH - 1] = 1.0;   // P_0 = newest value
    double base[MFX_NHIST];
    memcpy(base, prev, sizeof(base));
    for (int o = 1; o < NH; ++o) {
      double w[MFX_NHIST];
      lagrange_tail(ts, NH, NH - 1 - o, taus[tau], w);
      for (int j = 0; j < NH; ++j) cf.inc[tau][o - 1][j] = w[j] - prev[j];
      memcpy(prev, w, sizeof(prev));
      if (o == M.order[tau]) memcpy(base, w, sizeof(base));
    }
    // the polynomial of the order chosen at training for this prediction time
    for (int j = 0; j < NH; ++j) cf.base[tau][j] = base[j];
  }
  const double dlast = ts[NH - 1] - ts[NH - 2];
  for (int j = 0; j < NH - 2; ++j) cf.ratio[j] = (ts[j + 1] - ts[j]) / dlast;
  cf.ratio[NH - 2] = (tau1 - ts[NH - 1]) / dlast;
  memcpy(cf.fscale, M.fscale, sizeof(cf.fscale));
  memcpy(cf.tscale, M.tscale, sizeof(cf.tscale));
  float* X = mlp_input_buffer(M.mlp, M.E);
  launch_mfx_features(hz, cf, M.S, X, M.E, c.st);
  const float* Y = mlp_forward_on(M.mlp, M.E, c.st);
  launch_mfx_combine(hz, cf, Y, M.S, M.pred0, M.pred1, M.E, c.st);
  c.count(7);
}

// Push the half-step snapshot M.half at time th into the history ring.
void mfx_push_half(Ctx& c, MfxState& M, double th) {
  M.head = (M.head + 1) % MFX_NHIST;
  copy_dev(c, M.hist[M.head], M.half, M.E);
  M.thist[M.head] = th;
  M.nhist = std::min(M.nhist + 1, MFX_NHIST);
}

// One CMF2 attempt of length hdid from d_y (cmf2_base.f90:76-176); returns
// max(err_A, err_psi) / eps_int and leaves BHalf / psiHalf2 for cmf2_accept.
// ops_fresh: the operators and mean fields at d_y are already in place.
// The step-start Lanczos run works on the saved Krylov space (vectors and
// alpha/beta): the context's pointers are swapped for the scope.
struct KrylovScope {
  Ctx& c;
  cplx* k;
  double* l;
  KrylovScope(Ctx& cc, cplx* k0, double* l0) : c(cc), k(cc.d_krylov), l(cc.d_lan) {
    if (k0) {
      c.d_krylov = k0;
      c.d_lan = l0;
    }
  }
  ~KrylovScope() {
    c.d_krylov = k;
    c.d_lan = l;
  }
};

// The Krylov size at which a build from the same vector and operator stops for
// the step dt (lan_check's rule, cmf2_integration.f90:64-80) from the saved
// betas; 0 when they do not reach it.
int lan_reuse_count(const std::vector<double>& beta, double dt) {
  if (beta.empty()) return 0;
  double error = beta[0] * fabs(dt);
  for (int j = 2; j <= (int)beta.size(); ++j) {
    error = error * beta[j - 1] / (double)j * fabs(dt);
    if (error < EPS_B) return j;
  }
  return 0;
}

// after lan_finish of a step-start build: keep its betas for the retries
void lan_record(Ctx& c, CmfState& S) {
  if (!S.krylov0) return;
  const double* h_beta = c.h_scal + 64;
  S.beta0.assign(h_beta, h_beta + c.lan_nk);
  S.k0_valid = true;
}

double cmf2_attempt(Ctx& c, double t, double hdid, bool ops_fresh, bool reginv_done, bool ops_saved = false) {
  if (c.mixture)
    throw StatusError(MCTDH_EUNSUPPORTED, "CMF2 covers a single wave packet without dissipation (use rk45, dopri, abm or bs)");
  CmfState& S = cmf_state(c);
  const long long nA = c.naconftot;
  // With a second stream the regularised inverse of rho and the SPF half step
  // (which needs it) run beside the Lanczos build (which needs only h1mode).
  const bool overlap = c.st2 != nullptr;
  if (!ops_fresh && ops_saved && S.opE > 0) {
    // a retry from the same state: the step-start operators saved after their
    // evaluation (cmf2_base.f90:78-87 gives the same values again); rho^-1 MF as
    // in the evaluation (inside it without a second stream, below with one)
    copy_dev(c, c.d_in, c.d_y, c.ntot);
    launch_snap(S.opseg_d, (int)S.opseg_h.size(), S.opsave, S.opE, 1, c.st);
    c.count();
    if (!overlap) run_reginv(c);
    reginv_done = !overlap;
  } else if (!ops_fresh) {
    operators_and_mf(c, c.d_y, !overlap);           // cmf2_base.f90:78-87
    reginv_done = !overlap;
  }
  if (S.gwp) {
    // D0 = S^-1/2 (InverseSquareRootU, :63-73), Calc_DHD(DD0) (:87), B0 = D^H S A (:92)
    ProfScope ps(c, KP_GWP);
    launch_gwp_isqrt(S.isq_d, (int)S.isq_h.size(), c.d_status, c.st);
    launch_gwp_dhd(S.dhd0_d, (int)S.dhd0_h.size(), c.st);
    c.count(2);
    for (auto& b : S.a2b) run_prod(c, b);
  } else {
    copy_dev(c, S.B0, c.d_y, nA);                   // A_to_B: B = A without Gaussian modes
  }
  copy_dev(c, S.psiHalf, c.d_y, c.ntot);
  if (S.gwp) copy_dev(c, S.DDHalf, S.DD0, S.nD);
  // A retry from the same state (ops_saved) runs the step-start Lanczos on the
  // Krylov space of the rejected attempt's: the same B0 and operator give the
  // same vectors, alpha and beta, and a shorter step stops the build earlier, at
  // the size lan_reuse_count finds among the saved betas.
  const int nk_reuse = (ops_saved && S.k0_valid && S.krylov0) ? lan_reuse_count(S.beta0, 0.5 * hdid) : 0;
  if (!ops_saved) S.k0_valid = false;
  if (!overlap) {
    if (!reginv_done) run_reginv(c);
    {
      KrylovScope ks(c, S.krylov0, S.lan0);
      if (nk_reuse > 0) {
        LanRun L;
        L.nk = nk_reuse;
        lan_finish(c, L);
        lan_combine(c, S.BHalf, 0.5 * hdid);
      } else {
        lanczos(c, S.B0, S.BHalf, 0.5 * hdid, true);    // :97
        lan_record(c, S);
      }
    }
    propagate_spf_all(c, S, 0.5 * hdid, S.psiHalf, S.DDHalf);   // :109-115
  } else {
    KrylovScope ks(c, S.krylov0, S.lan0);
    // the Krylov build on c.st, the SPF integration (:109-115) on st2, in
    // lockstep: issue one step of each, wait for both, apply both controls
    CK(cudaEventRecord(c.ev_fork, c.st));
    CK(cudaStreamWaitEvent(c.st2, c.ev_fork, 0));
    LanRun L;
    L.B0 = S.B0;
    L.dt = 0.5 * hdid;
    SpfRun P;
    {
      StreamSwap sw(c, c.st2);
      if (!reginv_done) run_reginv(c);
      spf_begin(c, P, 0.5 * hdid, S.psiHalf, S.DDHalf);
    }
    bool lan_pending = false, spf_pending = false;
    if (nk_reuse > 0) {
      L.nk = nk_reuse;
    } else {
      lan_issue(c, L);
      lan_pending = true;
    }
    if (!P.finished) {
      StreamSwap sw(c, c.st2);
      spf_issue(c, S, P);
      spf_pending = true;
    }
    while (lan_pending || spf_pending) {
      if (lan_pending) CK(cudaStreamSynchronize(c.st));
      if (spf_pending) CK(cudaStreamSynchronize(c.st2));
      if (lan_pending) {
        lan_check(c, L);
        lan_pending = false;
        if (!L.done) {
          lan_issue(c, L);
          lan_pending = true;
        }
      }
      if (spf_pending) {
        StreamSwap sw(c, c.st2);
        spf_check(c, S, P);
        spf_pending = false;
        if (!P.finished) {
          spf_issue(c, S, P);
          spf_pending = true;
        }
      }
    }
    lan_finish(c, L);
    if (nk_reuse == 0) lan_record(c, S);
    lan_combine(c, S.BHalf, 0.5 * hdid);            // :97
    // the last SPF control's copies were issued on st2 after the last wait
    CK(cudaEventRecord(c.ev_join, c.st2));
    CK(cudaStreamWaitEvent(c.st, c.ev_join, 0));
    if (S.gwp) check_status(c);
  }
  if (S.gwp) {
    for (auto& b : S.b2a_half) run_prod(c, b);      // B_to_A(AHalf, BHalf, DDHalf)  :120
  } else {
    copy_dev(c, S.AHalf, S.BHalf, nA);
  }
  copy_dev(c, S.AHalf + nA, S.psiHalf + nA, c.dimpsi);
  MfxState* M = nullptr;
  auto it = g_mfx.find(&c);
  if (it != g_mfx.end()) M = it->second;
  operators_and_mf(c, S.AHalf);                     // :122-130
  if (M) snap_gather(c, *M, M->half);               // the extrapolator's history
  copy_dev(c, S.psiHalf2, c.d_y, c.ntot);
  if (S.gwp) copy_dev(c, S.DDHalf2, S.DD0, S.nD);
  propagate_spf_all(c, S, 0.5 * hdid, S.psiHalf2, S.DDHalf2);  // :132-141
  // err_psi = DeltaPsi(AHalf, psiHalf, AHalf, psiHalf2)  (:143): copies of both
  // states, then the overlaps on st2 beside the SPF sweep of :148-154 (read at the end)
  copy_dev(c, c.d_ovl1, S.AHalf, c.ntot);
  copy_dev(c, c.d_ovl2, S.AHalf, nA);
  copy_dev(c, c.d_ovl2 + nA, S.psiHalf2 + nA, c.dimpsi);
  if (overlap) {
    CK(cudaEventRecord(c.ev_fork, c.st));
    CK(cudaStreamWaitEvent(c.st2, c.ev_fork, 0));
    StreamSwap sw(c, c.st2);
    run_ovl(c, c.cmf_ovl);
  } else {
    run_ovl(c, c.cmf_ovl);
  }
  propagate_spf_all(c, S, 0.5 * hdid, S.psiHalf2, S.DDHalf2);  // :148-154
  h1_only(c, S.psiHalf2);                           // :158-163
  if (S.gwp) {
    launch_gwp_dhd(S.dhd2_d, (int)S.dhd2_h.size(), c.st);   // Calc_DHD(DDHalf2)  :164
    c.count();
  }
  lanczos(c, S.BHalf, S.B02, -0.5 * hdid, true);    // :169
  launch_axpy(S.B02, S.B0, mkc(-1, 0), nA, c.st);
  c.count();
  double err_A = sqrt(dot_now(c, S.B02, S.B02, nA).x) * 0.5;
  cplx o[3];
  {
    StreamSwap sw(c, overlap ? c.st2 : c.st);
    read_ovl(c, c.cmf_ovl, o);
  }
  const double err_psi = sqrt(fabs(2.0 * (1.0 - o[2].x / sqrt(o[0].x * o[1].x))));
  check_status(c);
  double error = std::max(err_A, err_psi) / c.eps_int;
  if (!std::isfinite(error)) throw StatusError(MCTDH_ENONFINITE, "non-finite CMF2 error estimate");
  return error;
}

// Accept: finish the coefficients with the reused Krylov space (:189) and update.
void cmf2_accept(Ctx& c, double hdid) {
  CmfState& S = cmf_state(c);
  if (S.gwp) {
    lanczos(c, S.BHalf, S.B02, 0.5 * hdid, false);
    for (auto& b : S.b2a_end) run_prod(c, b);       // B_to_A(A0, B0, DDHalf2)  :195
  } else {
    lanczos(c, S.BHalf, c.d_y, 0.5 * hdid, false);
  }
  copy_dev(c, c.d_y + c.naconftot, S.psiHalf2 + c.naconftot, c.dimpsi);
}

void cmf2(Ctx& c, double t, double htry, double* hdid_out, double* hnext_out, long long* tries) {
  if (c.mixture)
    throw StatusError(MCTDH_EUNSUPPORTED, "CMF2 covers a single wave packet without dissipation (use rk45, dopri, abm or bs)");
  MfxState* M = nullptr;
  auto it = g_mfx.find(&c);
  if (it != g_mfx.end()) M = it->second;
  const bool overlap = c.st2 != nullptr;
  // Step start: the operators and mean fields of d_y (cmf2_base.f90:78-87), or,
  // with an attached extrapolator and a full half-step history, h1mode computed
  // and rho / mean fields predicted (grid-mode models only).
  bool predicted = M && M->mlp && M->nhist == MFX_NHIST && c.modes_gwp.empty() && M->last_first_err < M->gate;
  double hdid = htry;
  for (;;) {
    if (predicted) {
      copy_dev(c, M->backup, c.d_y, c.ntot);
      mfx_predict(c, *M, t, t + 0.5 * hdid);
      // the density matrices are contracted exactly (their regularised inverse
      // would magnify a prediction error in the weakly occupied directions by up to
      // 1 / eps_rho^2); the mean fields come from the prediction
      copy_dev(c, c.d_in, c.d_y, c.naconftot);
      if (c.d_insplit) {
        launch_to_split(c.d_insplit, c.d_in, c.naconftot, c.st);
        c.count();
      }
      run_hole(c, c.rho_holes);
      run_red(c, c.red);
      launch_snap(M->segs_d, (int)M->segs_h.size(), M->pred0, M->E, 2, c.st);
      c.count();
      h1_only(c, c.d_y);
    } else {
      operators_and_mf(c, c.d_y, !overlap);
      if (M && M->recording) snap_gather(c, *M, M->start);
      // kept for the retries of a rejected attempt (same state, same operators)
      CmfState& S = cmf_state(c);
      if (S.opE > 0) {
        launch_snap(S.opseg_d, (int)S.opseg_h.size(), S.opsave, S.opE, 0, c.st);
        c.count();
      }
    }
    // reginv of the step start: done by operators_and_mf without a second stream;
    // otherwise inside the attempt, beside the Lanczos build
    const bool reginv_first = !predicted && !overlap;
    bool first = true;
    bool accepted_predicted = false;
    bool redo_plain = false;
    while (true) {
      ++*tries;
      if (*tries > 1000) throw StatusError(MCTDH_ESTEP, "CMF2 step not accepted after 1000 attempts");
      double error = 0.0;
      try {
        error = cmf2_attempt(c, t, hdid, first, first && reginv_first, !first && !predicted);
      } catch (const StatusError& e) {
        if (!(predicted && first) || (e.code != MCTDH_ENONFINITE && e.code != MCTDH_EEIG)) throw;
        // an extrapolated step start that made the SPF integration non-finite (or
        // its overlaps indefinite):
        // let both streams drain, then redo the step with the plain scheme
        CK(cudaStreamSynchronize(c.st));
        if (c.st2) CK(cudaStreamSynchronize(c.st2));
        redo_plain = true;
        break;
      }
      const bool was_predicted = predicted && first;
      if (M && first) M->last_first_err = error;
      first = false;
      if (M && M->log.size() < 5 * 100000) {
        const double row[5] = {t, hdid, error, was_predicted ? 1.0 : 0.0, -1.0};
        M->log.insert(M->log.end(), row, row + 5);
      }
      if (error > 1.0) {
        // rejected like any attempt; the retry recomputes the step-start mean fields
        if (was_predicted) ++M->rejected;
        hdid = hdid / sqrt(error) * 0.95;
        continue;
      }
      cmf2_accept(c, hdid);
      accepted_predicted = was_predicted;
      double hn = (error > 0.0) ? std::min(hdid / sqrt(error), hdid * 1.5) : hdid * 1.5;
      hn = std::min(hn, c.writetime);
      *hdid_out = hdid;
      *hnext_out = hn;
      break;
    }
    if (redo_plain) {
      ++M->fallbacks;
      copy_dev(c, c.d_y, M->backup, c.ntot);
      predicted = false;
      hdid = htry;
      continue;
    }
    if (accepted_predicted) {
      // the computed half-step mean fields against the extrapolation's prediction
      copy_dev(c, M->now, M->half, M->E);
      const double rel = snap_rel_diff(c, *M);
      M->last_rel = rel;
      if (!M->log.empty()) M->log.back() = rel;
      if (!(rel <= M->tol)) {
        // redo the step with the plain scheme
        ++M->fallbacks;
        copy_dev(c, c.d_y, M->backup, c.ntot);
        predicted = false;
        hdid = htry;
        continue;
      }
      ++M->mlp_steps;
    }
    if (M) {
      if (M->recording && !accepted_predicted) {
        std::vector<cplx> s0(M->E), sh(M->E);
        CK(cudaMemcpyAsync(s0.data(), M->start, sizeof(cplx) * M->E, cudaMemcpyDeviceToHost, c.st));
        CK(cudaMemcpyAsync(sh.data(), M->half, sizeof(cplx) * M->E, cudaMemcpyDeviceToHost, c.st));
        CK(cudaStreamSynchronize(c.st));
        M->rec_t0.push_back(t);
        M->rec_h.push_back(*hdid_out);
        M->rec_s0.insert(M->rec_s0.end(), s0.begin(), s0.end());
        M->rec_sh.insert(M->rec_sh.end(), sh.begin(), sh.end());
      }
      mfx_push_half(c, *M, t + 0.5 * *hdid_out);
    }
    return;
  }
}

// ---------------------------------------------------------------------------
// Context creation
// ---------------------------------------------------------------------------
// Vectors an ensemble provides to one of its members: views into the ensemble's
// contiguous state, input, output, stage and error vectors, and its stream.
struct MemberBufs {
  cplx *y, *y0, *in, *out, *k[7], *tmp, *err;
  cudaStream_t st;
};

Ctx* create(const mctdh_setup_t* s, const MemberBufs* mb = nullptr) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    throw StatusError(MCTDH_ECUDA, "no CUDA device available (this core has no CPU fallback)");
  Ctx* c = new Ctx();
  try {
    if (mb) {
      c->st = mb->st;
      c->own_stream = false;
      c->member = true;
      c->ar.chunk = (size_t)4 << 20;
    } else {
      CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
      CK(cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    }
    load_setup(*c, s);
    if (mb && c->mixture) throw StatusError(MCTDH_EUNSUPPORTED, "ensemble members are single wave packets without dissipation");
    c->d_status = (int*)c->ar.alloc(64);
    CK(cudaMemset(c->d_status, 0, 64));
    if (mb) {
      c->d_y = mb->y;
      c->d_y0 = mb->y0;
      c->d_in = mb->in;
      c->d_out = mb->out;
      for (int i = 0; i < 7; ++i) c->d_k[i] = mb->k[i];
      c->d_tmp = mb->tmp;
      c->d_err = mb->err;
    } else {
      c->d_y = c->ar.calloc_c(c->ntot);
      c->d_y0 = c->ar.calloc_c(c->ntot);
      c->d_in = c->ar.calloc_c(c->ntot);
      c->d_out = c->ar.calloc_c(c->ntot);
      for (int i = 0; i < 7; ++i) c->d_k[i] = c->ar.calloc_c(c->ntot);
      c->d_tmp = c->ar.calloc_c(c->ntot);
      c->d_err = c->ar.calloc_c(c->ntot);
    }
    c->d_scal = (double*)c->ar.alloc(4096);
    CK(cudaMallocHost(&c->h_scal, 4096));
    {
      const long long offs[2] = {0, c->ntot};
      c->d_off1 = (long long*)c->ar.alloc(sizeof(offs));
      CK(cudaMemcpy(c->d_off1, offs, sizeof(offs), cudaMemcpyHostToDevice));
    }
    plan_eom(*c);
    if (!mb && !c->mixture) {
      // CMF2 / Lanczos buffers (ensemble members, mixtures and dissipation integrate
      // with the derivative-based integrators only)
      c->d_hbin = c->ar.calloc_c(c->naconftot);
      if (c->hb_prec == 1) c->d_hbin32 = c->ar.calloc_c((c->naconftot + 1) / 2);
      {
        // block sums of the fused Lanczos dots (one per block of the 256-thread launches)
        const long long nb = (c->naconftot + 255) / 256;
        for (FusedDot* fd : {&c->hb_dot, &c->lan_nrm}) {
          fd->partial = c->ar.calloc_c(nb);
          fd->counter = (unsigned*)c->ar.alloc(sizeof(unsigned));
          CK(cudaMemset(fd->counter, 0, sizeof(unsigned)));
          fd->res = c->ar.calloc_c(1);
        }
        c->hb_dot.v = c->d_hbin;
        c->lan_nrm.v = c->d_hbin;   // any non-null vector requests the norm
      }
      c->d_hb = c->ar.calloc_c(c->naconftot);
      c->d_krylov = c->ar.calloc_c(c->naconftot * (NKRYLOV_MAX + 1));
      c->d_lan = (double*)c->ar.alloc(sizeof(double) * (3 * NKRYLOV_MAX + NKRYLOV_MAX * NKRYLOV_MAX));
      c->d_coef = c->ar.calloc_c(NKRYLOV_MAX);
      plan_hb(*c);
      c->d_ovl1 = c->ar.calloc_c(c->ntot);
      c->d_ovl2 = c->ar.calloc_c(c->ntot);
      plan_ovl(*c, c->cmf_ovl, c->d_ovl1, c->d_ovl2, (c->precision && c->eps_int >= 1e-5) ? 2 : 0, false, false);
    }
    // the compensated products of DeltaPsi (~1e-13) resolve 1 - Re<1|2>/.. ~ eps_int^2 / 2
    // only for loose tolerances; tight ones keep FP64
    plan_ovl(*c, c->dpsi_plan, c->d_tmp, c->d_err, (c->precision && c->eps_int >= 1e-5) ? 2 : 0);
    plan_ovl(*c, c->auto_plan, c->d_y0, c->d_y, 0);
    plan_ovl(*c, c->io_plan, c->d_in, c->d_out, 0);
    CK(cudaDeviceSynchronize());
  } catch (...) {
    if (c->st && c->own_stream) cudaStreamDestroy(c->st);
    delete c;
    throw;
  }
  return c;
}

template <typename F>
int64_t guarded(Ctx* c, F&& fn) {
  try {
    fn();
    return MCTDH_OK;
  } catch (const StatusError& e) {
    if (c) c->last_error = e.what();
    return e.code;
  } catch (const CudaError& e) {
    if (c) c->last_error = e.what();
    return MCTDH_ECUDA;
  } catch (const std::exception& e) {
    if (c) c->last_error = e.what();
    return MCTDH_EARG;
  }
}

// Host coefficient arrays are packet-major (APacketOffset(W) = W * nAConftot); the
// device keeps every state's packets together (one strided copy per state).
void upload(Ctx& c, cplx* dst, const double* A, const double* psi) {
  if (c.npk == 1) {
    CK(cudaMemcpyAsync(dst, A, sizeof(cplx) * c.naconftot, cudaMemcpyHostToDevice, c.st));
  } else {
    for (int s = 0; s < c.nstates; ++s)
      CK(cudaMemcpy2DAsync(dst + c.aoff[s], sizeof(cplx) * c.n1[s], reinterpret_cast<const cplx*>(A) + c.aoff1[s],
                           sizeof(cplx) * c.n1tot, sizeof(cplx) * c.n1[s], c.npk, cudaMemcpyHostToDevice, c.st));
  }
  if (c.dimpsi > 0)
    CK(cudaMemcpyAsync(dst + c.naconftot, psi, sizeof(cplx) * c.dimpsi, cudaMemcpyHostToDevice, c.st));
}
void download(Ctx& c, const cplx* src, double* A, double* psi) {
  if (c.npk == 1) {
    CK(cudaMemcpyAsync(A, src, sizeof(cplx) * c.naconftot, cudaMemcpyDeviceToHost, c.st));
  } else {
    for (int s = 0; s < c.nstates; ++s)
      CK(cudaMemcpy2DAsync(reinterpret_cast<cplx*>(A) + c.aoff1[s], sizeof(cplx) * c.n1tot, src + c.aoff[s],
                           sizeof(cplx) * c.n1[s], sizeof(cplx) * c.n1[s], c.npk, cudaMemcpyDeviceToHost, c.st));
  }
  if (c.dimpsi > 0)
    CK(cudaMemcpyAsync(psi, src + c.naconftot, sizeof(cplx) * c.dimpsi, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
}


// ---------------------------------------------------------------------------
// Ensembles of independent wavepackets of uneven shape (different state, mode,
// SPF and grid counts).  Every member is planned like a single context, on
// views into the ensemble's contiguous vectors; the members' descriptors are
// then concatenated, so each stage of the EOM (each chain depth, the
// contractions, the reduction, the regularised inverses, the term sums, the
// SPF derivatives) is ONE launch over all members.  Time stepping is adaptive
// RK in lockstep: a round runs one attempt of every member still stepping, each
// with its own step length, and the host applies each member's rkqs control
// (integrator.f90:36-91) to the round's error norms.
// ---------------------------------------------------------------------------
struct Ens {
  std::vector<Ctx*> m;
  std::vector<long long> off;   // member offsets in the ensemble vectors (size n + 1)
  long long total = 0;
  cudaStream_t st = nullptr;
  DevArena ar;
  cplx *Y = nullptr, *Y0 = nullptr, *IN = nullptr, *OUT = nullptr, *K[7] = {}, *TMP = nullptr, *ERR = nullptr;
  long long* off_d = nullptr;
  double* dt_d = nullptr;
  int* acc_d = nullptr;
  int* status_d = nullptr;
  cplx* res_d = nullptr;        // 3 per member: <1|1>, <2|2>, <1|2> of the error norm
  int precision = 0;
  cplx der = mkc(0, -1);
  double min_stepsize = 0, writetime = 0;
  // merged EOM plan
  std::vector<ProdBatch> chains, chains_full;
  ProdBatch gprods;
  HoleBatch rho_holes, holes;
  RedBatch red;
  std::vector<H1Desc> h1_h;
  H1Desc* h1_d = nullptr;
  int h1_maxn2 = 0;
  size_t h1_smem = 0;
  std::vector<MatSumDesc> msum_h;
  std::vector<MatSumSrc> msum_src_h;
  MatSumDesc* msum_d = nullptr;
  MatSumSrc* msum_src_d = nullptr;
  std::vector<RegInvDesc> reg_h;
  std::vector<MFOp> mfop_h;
  RegInvDesc* reg_d = nullptr;
  MFOp* mfop_d = nullptr;
  std::vector<SpfDesc> spf_h;
  std::vector<SpfOp> spfop_h;
  SpfDesc* spf_d = nullptr;
  SpfOp* spfop_d = nullptr;
  long long spf_tiles = 0;
  int spf_nf = 0;          // largest SPF count of the SPF derivative blocks and their operators
  std::vector<SumRange> sum_h;
  std::vector<SumSrc> src_h;
  SumRange* sum_d = nullptr;
  SumSrc* src_d = nullptr;
  // merged error-norm plan (DeltaPsi of every member)
  HoleBatch ov_spf_holes, ov_dots;
  RedBatch ov_spf_red, ov_dot_red;
  std::vector<ProdBatch> ov_chain;
  long long launches = 0, eom_count = 0, rounds = 0;
  std::string last_error;
  // CUDA graphs of the fixed launch sequences (index: 0 step-start derivative,
  // 1 Cash-Karp attempt round, 2 Dormand-Prince attempt round), with the launches
  // and EOM evaluations each replay stands for
  cudaGraphExec_t graph[3] = {nullptr, nullptr, nullptr};
  long long graph_launches[3] = {0, 0, 0}, graph_eoms[3] = {0, 0, 0};
  bool graphs_off = false;
  // autotuned launch shapes (ens_autotune): fibre tiles per contraction block,
  // block cap per contraction, tensor-core mode products (split path)
  bool tuned = false;
  int tune_tpb = HOLE_TPB, tune_cap = HOLE_CAP;
  bool tune_tc = true;
  double tune_ms = -1.0, tune_default_ms = -1.0;
  int tune_candidates = 0;
  // persistent CTAs of the merged mode products and contractions (0: one CTA per block)
  int persist_prod = 0, persist_hole = 0;
};

// Run `body` (launches on E.st only, no host synchronisation) as CUDA graph slot
// `k`: captured on the first call, replayed afterwards.  The round's step
// lengths are read from device memory, so one graph serves every round.  If
// capture fails the body runs eagerly from then on.
template <class F>
void ens_graph(Ens& E, int k, F body) {
  if (E.graphs_off) {
    body();
    return;
  }
  if (!E.graph[k]) {
    const long long l0 = E.launches, e0 = E.eom_count;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(E.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      E.graphs_off = true;
      body();
      return;
    }
    bool ok = true;
    try {
      body();
    } catch (...) {
      ok = false;
    }
    cudaError_t e = cudaStreamEndCapture(E.st, &g);
    cudaGraphExec_t ge = nullptr;
    ok = ok && e == cudaSuccess && g && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    E.graph_launches[k] = E.launches - l0;
    E.graph_eoms[k] = E.eom_count - e0;
    E.launches = l0;
    E.eom_count = e0;
    if (!ok) {
      cudaGetLastError();
      E.graphs_off = true;
      body();
      return;
    }
    E.graph[k] = ge;
  }
  CK(cudaGraphLaunch(E.graph[k], E.st));
  E.launches += E.graph_launches[k];
  E.eom_count += E.graph_eoms[k];
}

void merge_prod(ProdBatch& d, const ProdBatch& s) {
  d.h.insert(d.h.end(), s.h.begin(), s.h.end());
  d.prec = s.prec;
}
void merge_hole(HoleBatch& d, const HoleBatch& s) {
  d.h.insert(d.h.end(), s.h.begin(), s.h.end());
  d.prec = s.prec;
}
void merge_red(RedBatch& d, const RedBatch& s) {
  d.tg.insert(d.tg.end(), s.tg.begin(), s.tg.end());
  d.pending.insert(d.pending.end(), s.pending.begin(), s.pending.end());
}

Ens* ens_create(const mctdh_setup_t* setups, int n) {
  if (n < 1) throw StatusError(MCTDH_EARG, "empty ensemble");
  Ens* E = new Ens();
  try {
    CK(cudaStreamCreateWithFlags(&E->st, cudaStreamNonBlocking));
    // sizes first: the member layout fixes the ensemble vectors
    E->off.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      const mctdh_setup_t& s = setups[i];
      long long na = 0;
      for (int st = 0; st < s.nstates; ++st) {
        long long q = 1;
        for (int md = 0; md < s.nmodes; ++md) q *= s.nspf[md + s.nmodes * st];
        na += q;
      }
      E->off[i + 1] = E->off[i] + na + s.dimpsi;
    }
    E->total = E->off[n];
    E->Y = E->ar.calloc_c(E->total);
    E->Y0 = E->ar.calloc_c(E->total);
    E->IN = E->ar.calloc_c(E->total);
    E->OUT = E->ar.calloc_c(E->total);
    for (int j = 0; j < 7; ++j) E->K[j] = E->ar.calloc_c(E->total);
    E->TMP = E->ar.calloc_c(E->total);
    E->ERR = E->ar.calloc_c(E->total);
    for (int i = 0; i < n; ++i) {
      MemberBufs mb;
      const long long o = E->off[i];
      mb.y = E->Y + o;
      mb.y0 = E->Y0 + o;
      mb.in = E->IN + o;
      mb.out = E->OUT + o;
      for (int j = 0; j < 7; ++j) mb.k[j] = E->K[j] + o;
      mb.tmp = E->TMP + o;
      mb.err = E->ERR + o;
      mb.st = E->st;
      Ctx* c = create(&setups[i], &mb);
      E->m.push_back(c);
      if (c->ntot != E->off[i + 1] - o) throw StatusError(MCTDH_EARG, "member size mismatch");
      if (!c->modes_gwp.empty()) throw StatusError(MCTDH_EUNSUPPORTED, "ensembles of Gaussian-mode models");
      if (i == 0) {
        E->precision = c->precision;
        E->der = c->der;
        E->min_stepsize = c->min_stepsize;
        E->writetime = c->writetime;
      } else if (c->precision != E->precision || c->hole_prec != E->m[0]->hole_prec ||
                 c->mf_hole_prec != E->m[0]->mf_hole_prec || c->hb_prec != E->m[0]->hb_prec ||
                 c->der.x != E->der.x || c->der.y != E->der.y) {
        throw StatusError(MCTDH_EARG, "ensemble members must share precision and der_factor");
      }
      // merge the EOM plan
      if (E->chains.size() < c->chains.size()) E->chains.resize(c->chains.size());
      for (size_t dd = 1; dd < c->chains.size(); ++dd) merge_prod(E->chains[dd], c->chains[dd]);
      if (E->chains_full.size() < c->chains_full.size()) E->chains_full.resize(c->chains_full.size());
      for (size_t dd = 1; dd < c->chains_full.size(); ++dd) merge_prod(E->chains_full[dd], c->chains_full[dd]);
      merge_prod(E->gprods, c->gprods);
      merge_hole(E->rho_holes, c->rho_holes);
      merge_hole(E->holes, c->holes);
      merge_red(E->red, c->red);
      E->h1_h.insert(E->h1_h.end(), c->h1_h.begin(), c->h1_h.end());
      E->h1_maxn2 = std::max(E->h1_maxn2, c->h1_maxn2);
      E->h1_smem = std::max(E->h1_smem, c->h1_smem);
      for (MatSumDesc md : c->msum_h) {
        md.first += (int)E->msum_src_h.size();
        E->msum_h.push_back(md);
      }
      E->msum_src_h.insert(E->msum_src_h.end(), c->msum_src_h.begin(), c->msum_src_h.end());
      for (RegInvDesc rd : c->reg_h) {
        rd.op_first += (int)E->mfop_h.size();
        // no warm start in ensembles: the merged launches also refresh members that
        // are not stepping, so a member's call history would differ from its own
        // context's and its rounding with it
        rd.vprev = nullptr;
        rd.vcount = nullptr;
        E->reg_h.push_back(rd);
      }
      E->mfop_h.insert(E->mfop_h.end(), c->mfop_h.begin(), c->mfop_h.end());
      for (SpfDesc sd : c->spf_h) {
        sd.op_first += (int)E->spfop_h.size();
        sd.out_offset += o;
        sd.block_start = E->spf_tiles;
        E->spf_tiles += sd.ntile;
        E->spf_h.push_back(sd);
      }
      E->spfop_h.insert(E->spfop_h.end(), c->spfop_h.begin(), c->spfop_h.end());
      for (SumRange r : c->sum_h) {
        r.offset += o;
        r.first += (int)E->src_h.size();
        E->sum_h.push_back(r);
      }
      E->src_h.insert(E->src_h.end(), c->src_h.begin(), c->src_h.end());
      // merge the error-norm plan; its three results land at res_d + 3 i
      const OvlPlan& P = c->dpsi_plan;
      merge_hole(E->ov_spf_holes, P.spf_holes);
      merge_red(E->ov_spf_red, P.spf_red);
      if (E->ov_chain.size() < P.chain.size()) E->ov_chain.resize(P.chain.size());
      for (size_t dd = 1; dd < P.chain.size(); ++dd) merge_prod(E->ov_chain[dd], P.chain[dd]);
      merge_hole(E->ov_dots, P.dots);
      merge_red(E->ov_dot_red, P.dot_red);
    }
    E->res_d = E->ar.calloc_c(3LL * n);
    for (int i = 0; i < n; ++i)
      for (int q = 0; q < 3; ++q) E->ov_dot_red.tg[3 * i + q].out = E->res_d + 3 * i + q;
    for (auto& b : E->chains) b.finalize(E->ar);
    for (auto& b : E->chains_full) b.finalize(E->ar);
    E->gprods.finalize(E->ar);
    E->rho_holes.finalize(E->ar);
    E->holes.finalize(E->ar);
    E->red.finalize(E->ar);
    E->h1_d = upload_vec(E->ar, E->h1_h);
    E->msum_d = upload_vec(E->ar, E->msum_h);
    E->msum_src_d = upload_vec(E->ar, E->msum_src_h);
    E->reg_d = upload_vec(E->ar, E->reg_h);
    E->mfop_d = upload_vec(E->ar, E->mfop_h);
    E->spf_d = upload_vec(E->ar, E->spf_h);
    for (auto& x : E->spf_h) E->spf_nf = std::max(E->spf_nf, x.n);
    for (auto& x : E->spfop_h) E->spf_nf = std::max(E->spf_nf, x.n2);
    E->spfop_d = upload_vec(E->ar, E->spfop_h);
    E->sum_d = upload_vec(E->ar, E->sum_h);
    split_coeffs(E->src_h);
    E->src_d = upload_vec(E->ar, E->src_h);
    E->ov_spf_holes.finalize(E->ar);
    E->ov_spf_red.finalize(E->ar);
    for (auto& b : E->ov_chain) b.finalize(E->ar);
    E->ov_dots.finalize(E->ar);
    E->ov_dot_red.finalize(E->ar);
    E->off_d = upload_vec(E->ar, E->off);
    E->dt_d = (double*)E->ar.alloc(sizeof(double) * n);
    E->acc_d = (int*)E->ar.alloc(sizeof(int) * n);
    E->status_d = (int*)E->ar.alloc(64);
    CK(cudaMemset(E->status_d, 0, 64));
    if (E->h1_smem > 48 * 1024) throw StatusError(MCTDH_EUNSUPPORTED, "grid of a mode too large for the h1 kernel");
    CK(cudaDeviceSynchronize());
  } catch (...) {
    for (Ctx* c : E->m) delete c;
    if (E->st) cudaStreamDestroy(E->st);
    delete E;
    throw;
  }
  return E;
}

void ens_destroy(Ens* E) {
  cudaStreamSynchronize(E->st);
  for (auto& ge : E->graph)
    if (ge) cudaGraphExecDestroy(ge);
  for (Ctx* c : E->m) {
    for (auto& kv : c->dots) delete kv.second;
    for (auto e : c->evpool) cudaEventDestroy(e);
    delete c;
  }
  cudaStreamDestroy(E->st);
  delete E;
}

void ens_run_prod(Ens& E, const ProdBatch& b) {
  if (b.h.empty()) return;
  launch_prod(b.d, (int)b.h.size(), b.nblocks, b.maxn, E.st, b.prec, E.tune_tc ? 2 : 0, E.persist_prod);
  ++E.launches;
}
void ens_run_hole(Ens& E, const HoleBatch& b) {
  if (b.h.empty()) return;
  launch_hole(b.d, (int)b.h.size(), b.nblocks, E.st, b.prec, E.persist_hole);
  ++E.launches;
}
void ens_run_red(Ens& E, const RedBatch& b) {
  if (b.tg.empty()) return;
  launch_reduce(b.d_tg, (int)b.tg.size(), b.d_terms, E.st);
  ++E.launches;
}

// EOM of every member: IN -> out (same layout as the ensemble vectors).
void ens_eom(Ens& E, cplx* out) {
  launch_h1(E.h1_d, (int)E.h1_h.size(), E.h1_maxn2, E.h1_smem, true, E.st, E.precision);
  launch_matsum(E.msum_d, (int)E.msum_h.size(), E.msum_src_d, E.st);
  E.launches += 3;
  for (size_t i = 1; i < E.chains.size(); ++i) ens_run_prod(E, E.chains[i]);
  for (size_t i = 1; i < E.chains_full.size(); ++i) ens_run_prod(E, E.chains_full[i]);
  ens_run_prod(E, E.gprods);
  ens_run_hole(E, E.rho_holes);
  ens_run_hole(E, E.holes);
  ens_run_red(E, E.red);
  launch_reginv(E.reg_d, (int)E.reg_h.size(), E.mfop_d, E.status_d, E.st);
  launch_termsum(out, E.sum_d, (int)E.sum_h.size(), E.src_d, E.total, E.st, E.precision);
  launch_spf(E.spf_d, (int)E.spf_h.size(), E.spf_tiles, E.spfop_d, out, E.der, E.status_d, E.st, E.precision, E.spf_nf);
  E.launches += 5;
  E.eom_count++;
}

// Contraction tiling of every merged contraction batch and their reductions.
void ens_retile(Ens& E, int tpb, int cap) {
  for (HoleBatch* hb : {&E.rho_holes, &E.holes, &E.ov_spf_holes, &E.ov_dots}) hb->retile(tpb, cap, E.st);
  E.red.sync_nblk({&E.rho_holes, &E.holes}, E.st);
  E.ov_spf_red.sync_nblk({&E.ov_spf_holes}, E.st);
  E.ov_dot_red.sync_nblk({&E.ov_dots}, E.st);
}

// Autotuner of the ensemble's launch shapes, run once on the members' states
// before the first propagation (and before any graph is captured): each
// candidate (fibre tiles per contraction block, block cap per contraction, and
// in the split path tensor-core or CUDA-core mode products) is timed with CUDA
// events over two EOM evaluations of all members after one untimed one, and the
// fastest is kept.  The merged EOM and the error-norm contractions share the
// tiling.  Block counts change the order of the partial sums, not the
// arithmetic of a partial: results move at the rounding level only.
void ens_autotune(Ens& E) {
  if (E.tuned) return;
  E.tuned = true;
  struct Cand { int tpb, cap; bool tc; };
  std::vector<Cand> cands;
  const int tpbs[] = {8, 4, 16, 2};
  const int caps[] = {64, 128, 32};
  for (int tc = 1; tc >= 0; --tc) {
    if (!tc && E.precision != 1) break;
    for (int cap : caps)
      for (int tpb : tpbs) cands.push_back(Cand{tpb, cap, tc == 1});
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaMemcpyAsync(E.IN, E.Y, sizeof(cplx) * E.total, cudaMemcpyDeviceToDevice, E.st));
  const long long l0 = E.launches, q0 = E.eom_count;
  double best = 1e300;
  Cand bc = cands[0];
  for (size_t i = 0; i < cands.size(); ++i) {
    const Cand& c = cands[i];
    E.tune_tc = c.tc;
    ens_retile(E, c.tpb, c.cap);
    ens_eom(E, E.K[6]);
    CK(cudaEventRecord(e0, E.st));
    ens_eom(E, E.K[6]);
    ens_eom(E, E.K[6]);
    CK(cudaEventRecord(e1, E.st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (i == 0) E.tune_default_ms = 0.5 * ms;
    if (0.5 * ms < best) {
      best = 0.5 * ms;
      bc = c;
    }
  }
  // then, on the best tiling, persistent CTAs (q per SM for the 256-thread
  // contractions, 2q for the 128-thread mode products) against one CTA per block
  E.tune_tc = bc.tc;
  ens_retile(E, bc.tpb, bc.cap);
  int nsm = 0, dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int best_q = 0;
  for (int q : {2, 4}) {
    E.persist_prod = 2 * q * nsm;
    E.persist_hole = q * nsm;
    ens_eom(E, E.K[6]);
    CK(cudaEventRecord(e0, E.st));
    ens_eom(E, E.K[6]);
    ens_eom(E, E.K[6]);
    CK(cudaEventRecord(e1, E.st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    if (0.5 * ms < best) {
      best = 0.5 * ms;
      best_q = q;
    }
  }
  E.persist_prod = 2 * best_q * nsm;
  E.persist_hole = best_q * nsm;
  CK(cudaEventDestroy(e0));
  CK(cudaEventDestroy(e1));
  E.tune_tpb = bc.tpb;
  E.tune_cap = bc.cap;
  E.tune_ms = best;
  E.tune_candidates = (int)cands.size() + 2;
  E.launches = l0;
  E.eom_count = q0;
  // the EOMs of the tuning ran on the start states: clear what they may have flagged
  CK(cudaMemsetAsync(E.status_d, 0, sizeof(int), E.st));
  CK(cudaStreamSynchronize(E.st));
}

void ens_stage(Ens& E, cplx* out, const cplx* base, const double* coef, int nk) {
  StageArgs a;
  memset(&a, 0, sizeof(a));
  int n = 0;
  for (int j = 0; j < nk; ++j) {
    if (coef[j] == 0.0) continue;
    a.k[n] = E.K[j];
    a.c[n] = coef[j];
    ++n;
  }
  a.nk = n;
  launch_ens_stage(out, base, a, E.dt_d, E.off_d, (int)E.m.size(), E.total, E.st);
  ++E.launches;
}

void ens_check_status(Ens& E) {
  int st = 0;
  CK(cudaMemcpyAsync(&st, E.status_d, sizeof(int), cudaMemcpyDeviceToHost, E.st));
  CK(cudaStreamSynchronize(E.st));
  if (st != 0) {
    CK(cudaMemsetAsync(E.status_d, 0, sizeof(int), E.st));
    if (st & DEVST_EIG_NOCONV) throw StatusError(MCTDH_EEIG, "Jacobi eigensolver did not converge");
    if (st & DEVST_CHOL_FAIL) throw StatusError(MCTDH_EEIG, "SPF overlap matrix is not positive definite");
    throw StatusError(MCTDH_ENONFINITE, "device status " + std::to_string(st));
  }
}

// Every member from its time t[i] to tnext with adaptive RK (int_type 1 Cash-Karp,
// 2 Dormand-Prince); step[i]: the trial step, updated like propagate_wf's
// (propagator.f90:110-134).  Dormand-Prince re-evaluates the first stage at each
// step start instead of carrying it (the same numbers: the EOM is deterministic).
void ens_propagate(Ens& E, int method, double tnext, double* t, double* step) {
  ens_autotune(E);
  const int n = (int)E.m.size();
  const bool dp = (method == 2);
  const double errcon = pow(5.0 / RK_SAFETY, 1.0 / RK_PGROW);
  std::vector<int> done(n, 0), acc(n, 0);
  std::vector<double> dt(n, 0.0), hn(n, 0.0);
  std::vector<cplx> res(3 * (size_t)n);
  for (int i = 0; i < n; ++i) done[i] = (t[i] >= tnext - E.m[i]->min_stepsize);
  for (long long guard = 0;; ++guard) {
    bool any = false;
    for (int i = 0; i < n; ++i) any = any || !done[i];
    if (!any) break;
    if (guard > 1000000) throw StatusError(MCTDH_ESTEP, "ensemble propagation did not finish");
    // the derivative at every member's step start
    ens_graph(E, 0, [&] {
      CK(cudaMemcpyAsync(E.IN, E.Y, sizeof(cplx) * E.total, cudaMemcpyDeviceToDevice, E.st));
      ens_eom(E, E.K[0]);
    });
    std::vector<int> pending(n, 0);
    for (int i = 0; i < n; ++i) {
      pending[i] = !done[i];
      dt[i] = pending[i] ? step[i] : 0.0;
    }
    while (true) {
      bool anyp = false;
      for (int i = 0; i < n; ++i) anyp = anyp || pending[i];
      if (!anyp) break;
      ++E.rounds;
      std::vector<double> dth(n);
      for (int i = 0; i < n; ++i) dth[i] = pending[i] ? dt[i] : 0.0;
      CK(cudaMemcpyAsync(E.dt_d, dth.data(), sizeof(double) * n, cudaMemcpyHostToDevice, E.st));
      ens_graph(E, dp ? 2 : 1, [&] {
        for (int sg = 1; sg < 6; ++sg) {
          ens_stage(E, E.IN, E.Y, dp ? DP_B[sg] : CK_B[sg], sg);
          ens_eom(E, E.K[sg]);
        }
        ens_stage(E, E.TMP, E.Y, dp ? DP_C : CK_C, 6);
        if (dp) {
          CK(cudaMemcpyAsync(E.IN, E.TMP, sizeof(cplx) * E.total, cudaMemcpyDeviceToDevice, E.st));
          ens_eom(E, E.K[6]);
          ens_stage(E, E.ERR, E.Y, DP_D, 7);
        } else {
          ens_stage(E, E.ERR, E.Y, CK_D, 6);
        }
        // DeltaPsi (gmctdh_objects.f90:206-226) of every member
        ens_run_hole(E, E.ov_spf_holes);
        ens_run_red(E, E.ov_spf_red);
        for (size_t d = 1; d < E.ov_chain.size(); ++d) ens_run_prod(E, E.ov_chain[d]);
        ens_run_hole(E, E.ov_dots);
        ens_run_red(E, E.ov_dot_red);
      });
      CK(cudaMemcpyAsync(res.data(), E.res_d, sizeof(cplx) * 3 * n, cudaMemcpyDeviceToHost, E.st));
      ens_check_status(E);
      for (int i = 0; i < n; ++i) {
        acc[i] = 0;
        if (!pending[i]) continue;
        const Ctx& c = *E.m[i];
        const double o11 = res[3 * i].x, o22 = res[3 * i + 1].x, o12 = res[3 * i + 2].x;
        const double errmax = sqrt(fabs(2.0 * (1.0 - o12 / sqrt(o11 * o22)))) / c.eps_int;
        if (!std::isfinite(errmax)) throw StatusError(MCTDH_ENONFINITE, "non-finite RK error estimate");
        if (errmax < 1.0 || dt[i] <= c.min_stepsize) {   // rkqs accept (integrator.f90:63)
          double h = (errmax > errcon) ? RK_SAFETY * dt[i] * pow(errmax, RK_PGROW) : dt[i] * RK_MAXSCAL;
          h = std::max(h, c.min_stepsize);
          hn[i] = std::min(h, c.writetime);
          acc[i] = 1;
          pending[i] = 0;
        } else {
          double d = std::max(RK_MINSCAL * dt[i], RK_SAFETY * dt[i] * pow(errmax, RK_PSHRNK));
          dt[i] = std::max(d, c.min_stepsize);
        }
      }
      CK(cudaMemcpyAsync(E.acc_d, acc.data(), sizeof(int) * n, cudaMemcpyHostToDevice, E.st));
      launch_ens_accept(E.Y, E.TMP, E.acc_d, E.off_d, n, E.total, E.st);
      ++E.launches;
      for (int i = 0; i < n; ++i) {
        if (!acc[i]) continue;
        const Ctx& c = *E.m[i];
        t[i] += dt[i];
        if (t[i] >= tnext - c.min_stepsize) {
          done[i] = 1;
          continue;
        }
        const long long q = (long long)((tnext - t[i]) / hn[i]);   // propagator.f90:124-126
        step[i] = (q == 0) ? (tnext - t[i]) : (tnext - t[i]) / (double)(q + 1);
      }
    }
  }
  CK(cudaStreamSynchronize(E.st));
}

void observables(Ctx& c, double* energy, double* pop, double* norm, double* auto_re, double* auto_im);

}  // namespace

struct mctdh_ctx {
  Ctx* c;
};

// Error text for calls that run without a context (read with mctdh_last_error(NULL)).
void mctdh_set_global_error(const char* msg) { g_create_error = msg ? msg : ""; }

namespace {
// WriteOutput quantities (output.f90:35-87, 144-150) of the resident state.
void observables(Ctx& c, double* energy, double* pop, double* norm, double* auto_re, double* auto_im) {
  {
    c.skip_mult = true;
    try {
      eom_from(c, c.d_y, c.d_out);
    } catch (...) {
      c.skip_mult = false;
      throw;
    }
    c.skip_mult = false;
    // f * H A before the Gaussian-mode corrections (Calc_MeanField's energyMF); the
    // dissipative parts of the term sum are not energy
    const cplx* hA = c.modes_gwp.empty() ? c.d_out : c.d_adot;
    cplx e = dot_now(c, c.d_y, hA, c.naconftot);
    if (c.pk_xa) e = csub(e, dot_now(c, c.d_y, c.pk_xa, c.naconftot));
    if (c.pk_vmix) e = csub(e, dot_now(c, c.d_y, c.pk_vmix, c.naconftot));
    // energy = Re <A| H A> = Re( <A|dA> / der_factor )
    double dr = c.der.x, di = c.der.y, den = dr * dr + di * di;
    double en = (e.x * dr + e.y * di) / den;
    std::vector<double> p(c.nstates);
    double tot = 0.0;
    const int m0 = 0;
    for (int s = 0; s < c.nstates; ++s) {
      int n = c.m_of(m0, s);
      std::vector<cplx> r(n * n);
      CK(cudaMemcpyAsync(r.data(), c.rho[m0][s], sizeof(cplx) * n * n, cudaMemcpyDeviceToHost, c.st));
      CK(cudaStreamSynchronize(c.st));
      double tr = 0.0;
      if (c.is_gwp[m0]) {
        // Gaussian first mode: sum of rho o S00 from the upper triangle (output.f90:63-85)
        std::vector<cplx> S(n * n);
        const cplx* sp = c.s00[c.gwp_of[m0]][set_of(c, m0, s)][set_of(c, m0, s)];
        CK(cudaMemcpyAsync(S.data(), sp, sizeof(cplx) * n * n, cudaMemcpyDeviceToHost, c.st));
        CK(cudaStreamSynchronize(c.st));
        for (int j2 = 0; j2 < n; ++j2) {
          for (int j1 = 0; j1 < j2; ++j1) tr += 2.0 * cmul(r[j1 + n * j2], S[j1 + n * j2]).x;
          tr += cmul(r[j2 + n * j2], S[j2 + n * j2]).x;
        }
      } else {
        for (int j = 0; j < n; ++j) tr += r[j + n * j].x;
      }
      p[s] = tr;
      tot += tr;
    }
    run_ovl(c, c.auto_plan);
    cplx o[3];
    read_ovl(c, c.auto_plan, o);
    check_status(c);
    if (energy) *energy = en / tot;
    if (pop) for (int s = 0; s < c.nstates; ++s) pop[s] = p[s];
    if (norm) *norm = tot;
    if (auto_re) *auto_re = o[2].x;
    if (auto_im) *auto_im = o[2].y;
  }
}

// ---------------------------------------------------------------------------
// The rest of WriteOutput on the device: expectation values, natural
// populations, density matrices of the resident state (output.f90:88-140,
// 276-300, 449-500).
// ---------------------------------------------------------------------------
struct WriterPlan {
  bool expect_planned = false;
  std::vector<ProdBatch> chain;   // per term: prod_m h_m A_r, one batch per product depth
  HoleBatch dots;                 // <A_l | .>
  RedBatch red;                   // sum_t ae_t <..> per operator
  cplx* res = nullptr;
  std::vector<NatpopDesc> np_h;
  NatpopDesc* np_d = nullptr;
  double* np_out = nullptr;       // natpop | ggp | poperr
  long long np_len = 0, ggp_off = 0, perr_off = 0;
  int nspfmax = 0;
  std::map<int, cplx*> dens_scratch;     // dof -> Y (G x n) | DM (nG x nG)
  std::map<int, double*> dens_out;       // dof -> density | pop | trafo (per state: 2 nG, then nG^2)
};
std::map<const Ctx*, WriterPlan*> g_writer;

WriterPlan& writer_plan(Ctx& c) {
  WriterPlan*& W = g_writer[&c];
  if (!W) W = new WriterPlan();
  return *W;
}

// Expectation (output.f90:449-500): every mode's h1mode in mode order on A_r
// (identity matrices of grid modes are skipped, they change nothing; the
// Gaussian identity is S00), then <A_l| . > times ae_t summed per operator.
void plan_expect(Ctx& c, WriterPlan& W) {
  const int f = c.nmodes;
  W.res = c.ar.calloc_c(std::max(c.nexpect, 1));
  W.chain.assign(f + 1, ProdBatch());
  std::vector<HoleRef> refs;
  int g = 0;
  for (int i = 0; i < c.nexpect; ++i) {
    const int tg = W.red.add_target(W.res + i, 1, 1, 1, 0);
    for (int t = 0; t < c.exp_nterms[i]; ++t, ++g) {
      const int s1 = c.exp_lhs[g], s2 = c.exp_rhs[g];
      TRef cur;
      cur.p = c.d_in + c.aoff[s2];
      cur.shape = c.shape_of(s2);
      int depth = 0;
      for (int m = 0; m < f; ++m) {
        const int k = c.exp_ioper[m + f * g];
        if (!c.is_gwp[m] && c.is_identity[m + f * k]) continue;
        const int n1 = c.m_of(m, s1);
        std::vector<int> ns = cur.shape;
        ns[m] = n1;
        cplx* out = c.ar.calloc_c(prod_range(ns, 0, (int)ns.size()));
        ++depth;
        W.chain[depth].add(cur.p, out, c.hmat[m][k], n1, 0, cur.shape, m, n1, mkc(1, 0), 0);
        cur.p = out;
        cur.shape = ns;
      }
      if (prod_range(cur.shape, 0, (int)cur.shape.size()) != c.naconf[s1])
        throw StatusError(MCTDH_EARG, "expectation term does not map state r onto state l");
      const int h = W.dots.add(c.ar, c.d_in + c.aoff[s1], cur.p, c.naconf[s1], 1, 1, 1);
      refs.push_back(HoleRef{h, tg, c.exp_ae[g]});
    }
  }
  for (auto& b : W.chain) b.finalize(c.ar);
  W.dots.finalize(c.ar);
  for (auto& r : refs) W.red.add_term(r.target, W.dots.h[r.hole], r.alpha);
  W.red.finalize(c.ar);
  W.expect_planned = true;
}

void expectation(Ctx& c, cplx* values) {
  WriterPlan& W = writer_plan(c);
  if (!W.expect_planned) plan_expect(c, W);
  copy_dev(c, c.d_in, c.d_y, c.ntot);
  // h1mode of every operator on the resident SPFs, FP64 (Calc_h1mode before
  // WriteOutput, output.f90:35-41)
  if (!c.modes_gwp.empty()) {
    launch_gwp_ovl(c.gs_d, (int)c.gs_h.size(), c.st);
    launch_gwp_h1(c.gh1_d, (int)c.gh1_h.size(), c.st);
    launch_gwp_h1(c.xgh1_d, (int)c.xgh1_h.size(), c.st);
    c.count(3);
  }
  launch_h1(c.h1_d, (int)c.h1_h.size(), c.h1_maxn2, c.h1_smem, true, c.st, 0);
  launch_h1(c.xh1_d, (int)c.xh1_h.size(), c.h1_maxn2, c.h1_smem, true, c.st, 0);
  c.count(2);
  for (size_t i = 1; i < W.chain.size(); ++i) run_prod(c, W.chain[i]);
  run_hole(c, W.dots);
  run_red(c, W.red);
  CK(cudaMemcpyAsync(values, W.res, sizeof(cplx) * c.nexpect, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  check_status(c);
}

// Calc_Density (output.f90:332-445) along one DOF for every state.
void density(Ctx& c, int dof, const double* trafo, int ldt, double xmin, double xmax, double* dens, double* pop) {
  WriterPlan& W = writer_plan(c);
  int mode = -1, k = -1;
  for (int m = 0; m < c.nmodes && mode < 0; ++m)
    for (int q = 0; q < c.nmodedof[m]; ++q)
      if (c.mode_dofs[m][q] == dof) { mode = m; k = q; }
  if (mode < 0) throw StatusError(MCTDH_EARG, "dof not in any mode");
  const int nG = c.ngp[dof];
  if (nG < 2) throw StatusError(MCTDH_EARG, "density needs at least two grid points");
  const bool gwp = c.is_gwp[mode];
  if (!W.dens_out.count(dof)) {
    W.dens_out[dof] = (double*)c.ar.alloc(sizeof(double) * (2LL * nG * c.nstates + (long long)nG * nG));
    if (!gwp) {
      int nmax = 0;
      for (int s = 0; s < c.nstates; ++s) nmax = std::max(nmax, c.m_of(mode, s));
      W.dens_scratch[dof] = c.ar.calloc_c((long long)c.gmode[mode] * nmax + (long long)nG * nG);
    }
  }
  double* out = W.dens_out[dof];
  double* d_trafo = out + 2LL * nG * c.nstates;
  const bool with_pop = !gwp && trafo && pop;
  if (with_pop) {
    if (ldt < nG) throw StatusError(MCTDH_EARG, "trafo leading dimension below ngp");
    for (int b = 0; b < nG; ++b)
      CK(cudaMemcpyAsync(d_trafo + (long long)nG * b, trafo + (long long)ldt * b, sizeof(double) * nG,
                         cudaMemcpyHostToDevice, c.st));
  }
  operators_and_mf(c, c.d_y);   // rho of the resident state (output.f90:35-41)
  for (int s = 0; s < c.nstates; ++s) {
    const int n = c.m_of(mode, s);
    double* ds = out + (long long)nG * s;
    double* ps = out + (long long)nG * (c.nstates + s);
    if (gwp) {
      const int i = c.gwp_of[mode];
      DensGwpArgs a;
      memset(&a, 0, sizeof(a));
      a.xi = psi_block(c, c.d_y, mode, s);
      a.a = c.gwpa_d + (size_t)c.gwp_lda * c.ns00max * i;
      a.rho = c.rho[mode][s];
      a.dens = ds;
      a.x0 = xmin;
      a.delta = (xmax - xmin) / (double)(nG - 1);
      a.n = n;
      a.nmd = c.nmodedof[mode];
      a.lda = c.gwp_lda;
      a.k = k;
      a.nG = nG;
      launch_density_gwp(a, c.st);
    } else {
      DensGridArgs a;
      memset(&a, 0, sizeof(a));
      int ll = 1, nl = 1;
      for (int q = 0; q < k; ++q) ll *= c.ngp[c.mode_dofs[mode][q]];
      for (int q = k + 1; q < c.nmodedof[mode]; ++q) nl *= c.ngp[c.mode_dofs[mode][q]];
      a.phi = psi_block(c, c.d_y, mode, s);
      a.rho = c.rho[mode][s];
      a.Y = W.dens_scratch[dof];
      a.DM = W.dens_scratch[dof] + (long long)c.gmode[mode] * n;
      a.trafo = with_pop ? d_trafo : nullptr;
      a.ldt = nG;
      a.dens = ds;
      a.pop = ps;
      a.n = n;
      a.nG = nG;
      a.ll = ll;
      a.nl = nl;
      launch_density_grid(a, c.st);
    }
    c.count();
  }
  CK(cudaMemcpyAsync(dens, out, sizeof(double) * nG * c.nstates, cudaMemcpyDeviceToHost, c.st));
  if (with_pop)
    CK(cudaMemcpyAsync(pop, out + (long long)nG * c.nstates, sizeof(double) * nG * c.nstates,
                       cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  check_status(c);
}

void plan_natpop(Ctx& c, WriterPlan& W) {
  const int f = c.nmodes, ng = (int)c.modes_gwp.size();
  for (int m = 0; m < f; ++m)
    for (int s = 0; s < c.nstates; ++s) W.nspfmax = std::max(W.nspfmax, c.m_of(m, s));
  const long long nnat = (long long)W.nspfmax * f * c.nstates;
  const long long ngg = (long long)std::max(c.ns00max, 1) * ng * c.nstates;
  W.ggp_off = nnat;
  W.perr_off = nnat + ngg;
  W.np_len = nnat + 2 * ngg;
  W.np_out = (double*)c.ar.alloc(sizeof(double) * std::max(W.np_len, 1LL));
  for (int s = 0; s < c.nstates; ++s) {
    for (int m = 0; m < f; ++m) {
      NatpopDesc d;
      memset(&d, 0, sizeof(d));
      d.n = c.m_of(m, s);
      d.rho = c.rho[m][s];
      d.natpop = W.np_out + (long long)W.nspfmax * (m + f * s);
      if (c.is_gwp[m]) {
        const int i = c.gwp_of[m];
        d.S = c.s00[i][set_of(c, m, s)][set_of(c, m, s)];
        d.work = c.ar.calloc_c(2LL * d.n * d.n);
        d.ggp = W.np_out + W.ggp_off + (long long)c.ns00max * (i + ng * s);
        d.poperr = W.np_out + W.perr_off + (long long)c.ns00max * (i + ng * s);
      }
      W.np_h.push_back(d);
    }
  }
  W.np_d = upload_vec(c.ar, W.np_h);
}

void natpop(Ctx& c, double* nat, double* ggp, double* poperr) {
  WriterPlan& W = writer_plan(c);
  if (!W.np_d) plan_natpop(c, W);
  operators_and_mf(c, c.d_y);   // rho and S00 of the resident state (output.f90:35-41)
  CK(cudaMemsetAsync(W.np_out, 0, sizeof(double) * W.np_len, c.st));
  launch_natpop(W.np_d, (int)W.np_h.size(), c.d_status, c.st);
  c.count();
  const long long nnat = W.ggp_off, ngg = W.perr_off - W.ggp_off;
  CK(cudaMemcpyAsync(nat, W.np_out, sizeof(double) * nnat, cudaMemcpyDeviceToHost, c.st));
  if (ggp && ngg > 0 && !c.modes_gwp.empty())
    CK(cudaMemcpyAsync(ggp, W.np_out + W.ggp_off, sizeof(double) * ngg, cudaMemcpyDeviceToHost, c.st));
  if (poperr && ngg > 0 && !c.modes_gwp.empty())
    CK(cudaMemcpyAsync(poperr, W.np_out + W.perr_off, sizeof(double) * ngg, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  check_status(c);
}
}  // namespace

struct mctdh_ens {
  Ens* e;
};

template <typename F>
int64_t ens_guarded(mctdh_ens* h, F&& fn) {
  try {
    fn();
    return MCTDH_OK;
  } catch (const StatusError& e) {
    h->e->last_error = e.what();
    return e.code;
  } catch (const CudaError& e) {
    h->e->last_error = e.what();
    return MCTDH_ECUDA;
  } catch (const std::exception& e) {
    h->e->last_error = e.what();
    return MCTDH_EARG;
  }
}

extern "C" {

int64_t mctdh_create(const mctdh_setup_t* setup, mctdh_ctx_t** out) {
  if (!setup || !out) return MCTDH_EARG;
  *out = nullptr;
  try {
    Ctx* c = create(setup);
    if (tc_enabled()) tc_prepare();
    *out = new mctdh_ctx{c};
    g_create_error.clear();
    return MCTDH_OK;
  } catch (const StatusError& e) {
    g_create_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_create_error = e.what();
    return MCTDH_ECUDA;
  }
}

int64_t mctdh_destroy(mctdh_ctx_t* ctx) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  cudaStreamSynchronize(c->st);
  if (c->st2) cudaStreamSynchronize(c->st2);
  auto it = g_cmf.find(c);
  if (it != g_cmf.end()) {
    delete it->second;
    g_cmf.erase(it);
  }
  auto mi = g_mfx.find(c);
  if (mi != g_mfx.end()) {
    delete mi->second;
    g_mfx.erase(mi);
  }
  auto wi = g_writer.find(c);
  if (wi != g_writer.end()) {
    delete wi->second;
    g_writer.erase(wi);
  }
  for (auto& kv : c->dots) delete kv.second;
  drain_profile(*c);
  for (auto e : c->evpool) cudaEventDestroy(e);
  for (auto e : c->user_ev) if (e) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->st);
  delete c;
  delete ctx;
  return MCTDH_OK;
}

const char* mctdh_last_error(mctdh_ctx_t* ctx) {
  if (!ctx) return g_create_error.c_str();
  return ctx->c->last_error.c_str();
}

int64_t mctdh_launch_count(mctdh_ctx_t* ctx) { return ctx ? ctx->c->launches : 0; }

int64_t mctdh_calc_derivs(mctdh_ctx_t* ctx, const double* A, const double* psi, double* dA, double* dpsi,
                          double t) {
  if (!ctx || !A || !psi || !dA || !dpsi) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    (void)t;
    upload(*c, c->d_in, A, psi);
    eom(*c, c->d_out);
    check_status(*c);
    download(*c, c->d_out, dA, dpsi);
  });
}

int64_t mctdh_set_state(mctdh_ctx_t* ctx, const double* A, const double* psi, int64_t as_start) {
  if (!ctx || !A || !psi) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_y, A, psi);
    c->fsal_valid = false;
    c->ad_valid = false;
    c->bs_tnew = -1e16;   // SetupBS and propagator.f90:213: a new propagation
    c->bs_hnext = -1e15;
    c->ops_fresh = false;
    auto mi = g_mfx.find(c);
    if (mi != g_mfx.end()) mi->second->nhist = 0;
    if (as_start) copy_dev(*c, c->d_y0, c->d_y, c->ntot);
    CK(cudaStreamSynchronize(c->st));
  });
}

int64_t mctdh_get_state(mctdh_ctx_t* ctx, double* A, double* psi) {
  if (!ctx || !A || !psi) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] { download(*c, c->d_y, A, psi); });
}

int64_t mctdh_rkqs(mctdh_ctx_t* ctx, double* A, double* psi, double* dA, double* dpsi, double t, double htry,
                   double* hdid, double* hnext, int64_t method) {
  if (!ctx || !A || !psi || !dA || !dpsi || !hdid || !hnext) return MCTDH_EARG;
  if (method != 1 && method != 2) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_y, A, psi);
    upload(*c, c->d_k[0], dA, dpsi);
    long long att = 0;
    rkqs(*c, t, htry, hdid, hnext, (int)method, &att);
    download(*c, c->d_y, A, psi);
    if (method == 2) download(*c, c->d_k[0], dA, dpsi);
  });
}

int64_t mctdh_rk_attempt(mctdh_ctx_t* ctx, double* A, double* psi, double* dA, double* dpsi, double t,
                         double dt, int64_t method, double* errmax) {
  if (!ctx || !A || !psi || !dA || !dpsi || !errmax) return MCTDH_EARG;
  if (method != 1 && method != 2) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_y, A, psi);
    upload(*c, c->d_k[0], dA, dpsi);
    *errmax = rk_attempt(*c, t, dt, (int)method);
    download(*c, c->d_tmp, A, psi);
    if (method == 2) download(*c, c->d_k[6], dA, dpsi);
  });
}

int64_t mctdh_cmf2_attempt(mctdh_ctx_t* ctx, double* A, double* psi, double t, double h, double* error) {
  if (!ctx || !A || !psi || !error) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_y, A, psi);
    c->ops_fresh = false;
    *error = cmf2_attempt(*c, t, h, false, false);
    cmf2_accept(*c, h);
    download(*c, c->d_y, A, psi);
  });
}

int64_t mctdh_cmf2(mctdh_ctx_t* ctx, double* A, double* psi, double t, double htry, double* hdid,
                   double* hnext) {
  if (!ctx || !A || !psi || !hdid || !hnext) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_y, A, psi);
    long long tries = 0;
    cmf2(*c, t, htry, hdid, hnext, &tries);
    download(*c, c->d_y, A, psi);
  });
}

int64_t mctdh_propagate(mctdh_ctx_t* ctx, int64_t int_type, double tnext, double* t, double* step,
                        int64_t* nsteps, int64_t* nattempts, int64_t* neom) {
  if (!ctx || !t || !step) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    long long steps = 0, att = 0;
    long long eom0 = c->eom_count;
    double time = *t, stepsize = *step;
    while (true) {
      double sdone, snext;
      if (int_type == 4) {
        bs_step(*c, time, stepsize, &sdone, &snext);
        ++att;
        ++steps;
        time += sdone;
        if (time >= tnext - c->min_stepsize) break;
        long long q = (long long)((tnext - time) / snext);
        stepsize = (q == 0) ? (tnext - time) : (tnext - time) / (double)(q + 1);
        continue;
      }
      if (int_type == 3) {
        const bool boot = adams_or_boot_step(*c, time, stepsize, &sdone, &snext, &att);
        ++steps;
        time += sdone;
        if (boot) {
          if (time >= tnext - c->min_stepsize) break;
          long long q = (long long)((tnext - time) / snext);
          stepsize = (q == 0) ? (tnext - time) : (tnext - time) / (double)(q + 1);
        } else {
          if (time >= tnext) break;   // propagator.f90:191-193
          stepsize = std::min((tnext - time) / (double)((long long)((tnext - time) / snext) + 1), tnext - time);
        }
        continue;
      }
      if (int_type == 10) {
        cmf2(*c, time, stepsize, &sdone, &snext, &att);
      } else if (int_type == 1 || int_type == 2) {
        if (int_type == 1 || !c->fsal_valid) {
          // propagator.f90:116 (Cash-Karp).  Dormand-Prince reuses the last stage
          // (FSAL); its very first derivative is evaluated here, where the reference
          // reads a never-computed dAVector (propagator.f90:98, integrator.f90:187).
          eom_from(*c, c->d_y, c->d_k[0]);
        }
        rkqs(*c, time, stepsize, &sdone, &snext, (int)int_type, &att);
        c->fsal_valid = (int_type == 2);
      } else {
        throw StatusError(MCTDH_EUNSUPPORTED, "integrator type not supported");
      }
      ++steps;
      time += sdone;
      if (time >= tnext - c->min_stepsize) break;
      long long q = (long long)((tnext - time) / snext);
      stepsize = (q == 0) ? (tnext - time) : (tnext - time) / (double)(q + 1);
    }
    CK(cudaStreamSynchronize(c->st));
    *t = time;
    *step = stepsize;
    if (nsteps) *nsteps = steps;
    if (nattempts) *nattempts = att;
    if (neom) *neom = c->eom_count - eom0;
  });
}

int64_t mctdh_step(mctdh_ctx_t* ctx, int64_t int_type, double t, double htry, double* hdid, double* hnext,
                   int64_t* nattempts) {
  if (!ctx || !hdid || !hnext) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    long long att = 0;
    if (int_type == 3) {
      adams_or_boot_step(*c, t, htry, hdid, hnext, &att);
    } else if (int_type == 4) {
      bs_step(*c, t, htry, hdid, hnext);
      att = 1;
    } else if (int_type == 10) {
      cmf2(*c, t, htry, hdid, hnext, &att);
    } else if (int_type == 1 || int_type == 2) {
      if (int_type == 1 || !c->fsal_valid) eom_from(*c, c->d_y, c->d_k[0]);
      rkqs(*c, t, htry, hdid, hnext, (int)int_type, &att);
      c->fsal_valid = (int_type == 2);
    } else {
      throw StatusError(MCTDH_EUNSUPPORTED, "integrator type not supported");
    }
    if (nattempts) *nattempts = att;
  });
}

int64_t mctdh_mfx_size(mctdh_ctx_t* ctx, int64_t* E) {
  if (!ctx || !E) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] { *E = mfx_state(*c).E; });
}

int64_t mctdh_mfx_record(mctdh_ctx_t* ctx, int64_t enable) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    MfxState& M = mfx_state(*c);
    if (enable == 2 || enable == 0) {
      M.rec_t0.clear();
      M.rec_h.clear();
      M.rec_s0.clear();
      M.rec_sh.clear();
    }
    M.recording = enable != 0;
  });
}

int64_t mctdh_mfx_fetch(mctdh_ctx_t* ctx, int64_t maxrec, double* t0, double* h, double* snap0, double* snaphalf,
                        int64_t* n) {
  if (!ctx || !n) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    MfxState& M = mfx_state(*c);
    const long long nr = (long long)M.rec_t0.size();
    *n = nr;
    const long long k = std::min<long long>(nr, maxrec);
    for (long long i = 0; i < k; ++i) {
      if (t0) t0[i] = M.rec_t0[i];
      if (h) h[i] = M.rec_h[i];
    }
    if (snap0) memcpy(snap0, M.rec_s0.data(), sizeof(cplx) * M.E * k);
    if (snaphalf) memcpy(snaphalf, M.rec_sh.data(), sizeof(cplx) * M.E * k);
  });
}

int64_t mctdh_mfx_attach(mctdh_ctx_t* ctx, mctdh_mlp* mlp, const double* fscale, const double* tscale, double tol) {
  if (!ctx) return MCTDH_EARG;
  if (mlp && (!fscale || !tscale)) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    if (mlp && !mlp_has_shape(mlp, MFX_NFEAT, MFX_NOUT))
      throw StatusError(MCTDH_EARG, "the network must map 20 inputs to 4 outputs");
    if (mlp && !c->modes_gwp.empty())
      throw StatusError(MCTDH_EUNSUPPORTED, "the mean-field extrapolator covers grid-mode models only");
    MfxState& M = mfx_state(*c);
    M.mlp = mlp;
    if (mlp) {
      for (int j = 0; j < MFX_NFEAT; ++j) {
        if (!(fscale[j] > 0.0)) throw StatusError(MCTDH_EARG, "input scales must be positive");
        M.fscale[j] = fscale[j];
      }
      for (int j = 0; j < MFX_NOUT; ++j) M.tscale[j] = tscale[j];
    }
    M.tol = tol;
  });
}

int64_t mctdh_mfx_orders(mctdh_ctx_t* ctx, int64_t order_start, int64_t order_half) {
  if (!ctx || order_start < 1 || order_start > MFX_NHIST - 1 || order_half < 1 || order_half > MFX_NHIST - 1)
    return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    MfxState& M = mfx_state(*c);
    M.order[0] = (int)order_start;
    M.order[1] = (int)order_half;
  });
}

int64_t mctdh_mfx_gate(mctdh_ctx_t* ctx, double gate) {
  if (!ctx || !(gate > 0.0)) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] { mfx_state(*c).gate = gate; });
}

int64_t mctdh_mfx_predict(mctdh_ctx_t* ctx, const double* hist, const double* ts, double tau0, double tau1,
                          double* out0, double* out1) {
  if (!ctx || !hist || !ts || !out0 || !out1) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    MfxState& M = mfx_state(*c);
    if (!M.mlp) throw StatusError(MCTDH_EARG, "no extrapolator attached");
    for (int j = 0; j < MFX_NHIST; ++j) {
      CK(cudaMemcpyAsync(M.hist[j], hist + 2 * M.E * j, sizeof(cplx) * M.E, cudaMemcpyHostToDevice, c->st));
      M.thist[j] = ts[j];
    }
    M.head = MFX_NHIST - 1;
    M.nhist = MFX_NHIST;
    mfx_predict(*c, M, tau0, tau1);
    CK(cudaMemcpyAsync(out0, M.pred0, sizeof(cplx) * M.E, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(out1, M.pred1, sizeof(cplx) * M.E, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    M.nhist = 0;
  });
}

int64_t mctdh_mfx_log(mctdh_ctx_t* ctx, int64_t maxrows, double* rows, int64_t* n) {
  if (!ctx || !n) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    MfxState& M = mfx_state(*c);
    const long long nr = (long long)M.log.size() / 5;
    *n = nr;
    if (rows) memcpy(rows, M.log.data(), sizeof(double) * 5 * std::min<long long>(nr, maxrows));
  });
}

int64_t mctdh_mfx_stats(mctdh_ctx_t* ctx, int64_t* mlp_steps, int64_t* fallbacks, int64_t* rejected,
                        double* last_rel) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    MfxState& M = mfx_state(*c);
    if (mlp_steps) *mlp_steps = M.mlp_steps;
    if (fallbacks) *fallbacks = M.fallbacks;
    if (rejected) *rejected = M.rejected;
    if (last_rel) *last_rel = M.last_rel;
  });
}

int64_t mctdh_counters(mctdh_ctx_t* ctx, int64_t* launches, int64_t* eom, int64_t* hb) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  if (launches) *launches = c->launches;
  if (eom) *eom = c->eom_count;
  if (hb) *hb = c->hb_count;
  return MCTDH_OK;
}

int64_t mctdh_fp64_peak(double* tflops) {
  if (!tflops) return MCTDH_EARG;
  *tflops = measure_fp64_tflops();
  return *tflops > 0 ? MCTDH_OK : MCTDH_ECUDA;
}

int64_t mctdh_event_record(mctdh_ctx_t* ctx, int64_t slot) {
  if (!ctx || slot < 0 || slot >= 16) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    if (!c->user_ev[slot]) CK(cudaEventCreate(&c->user_ev[slot]));
    CK(cudaEventRecord(c->user_ev[slot], c->st));
  });
}

int64_t mctdh_event_elapsed(mctdh_ctx_t* ctx, int64_t s0, int64_t s1, double* ms) {
  if (!ctx || !ms || s0 < 0 || s1 < 0 || s0 >= 16 || s1 >= 16) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    if (!c->user_ev[s0] || !c->user_ev[s1]) throw StatusError(MCTDH_EARG, "event slot not recorded");
    CK(cudaEventSynchronize(c->user_ev[s1]));
    float f = 0;
    CK(cudaEventElapsedTime(&f, c->user_ev[s0], c->user_ev[s1]));
    *ms = f;
  });
}

int64_t mctdh_timing(mctdh_ctx_t* ctx, int64_t mode) {
  if (!ctx || mode < 0 || mode > 2) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    drain_timing(*c);
    if (mode == 2) {
      for (int i = 0; i < 8; ++i) {
        c->rt_ms[i] = 0.0;
        c->rt_calls[i] = 0;
      }
    }
    c->timing = mode != 0;
  });
}

int64_t mctdh_timing_read(mctdh_ctx_t* ctx, int64_t timer, int64_t* calls, double* ms) {
  if (!ctx || timer < 1 || timer > 8) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    drain_timing(*c);
    if (calls) *calls = c->rt_calls[timer - 1];
    if (ms) *ms = c->rt_ms[timer - 1];
  });
}

// The `timing` file of write_timings (timingmod.f90:72-103): total wall time,
// then per routine the calls, ms per call, minutes and % of the wall time, with
// the routine times measured on the device.
int64_t mctdh_write_timings(mctdh_ctx_t* ctx, const char* path, double walltime_s) {
  if (!ctx || !path || !(walltime_s > 0.0)) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    drain_timing(*c);
    static const char* names[8] = {"CalcDerivs",  "normWF/wf_ovl",    "Calc_MeanField",   "Calc_CY",
                                   "Calc_h1mode", "Calc_Der_SPF_DVR", "Calc_Der_SPF_GWP", "Lanczos"};
    FILE* fp = fopen(path, "w");
    if (!fp) throw StatusError(MCTDH_EARG, std::string("cannot open ") + path);
    const int h = (int)(walltime_s / 3600.0);
    const int m = (int)((walltime_s - h * 3600.0) / 60.0);
    const int sec = (int)(walltime_s - h * 3600.0 - m * 60.0);
    fprintf(fp, "Total time:   %d h   %d m   %d s\n \n \n", h, m, sec);
    fprintf(fp, "          Subroutine    Calls N    time/N [ms]      time [min]    %%time\n \n");
    for (int i = 0; i < 8; ++i) {
      const long long n = c->rt_calls[i];
      const double sub = c->rt_ms[i] * 1e-3;
      const double per = n > 0 ? sub / (double)n * 1000.0 : 0.0;
      fprintf(fp, "%20s    %7lld   %9.2f   %11.2f      %6.2f\n", names[i], n, per, sub / 60.0, sub / walltime_s * 100.0);
    }
    fclose(fp);
  });
}

int64_t mctdh_profile(mctdh_ctx_t* ctx, int64_t enable) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    drain_profile(*c);
    if (enable == 2) for (auto& k : c->prof) k = KProf();
    c->profiling = enable != 0;
  });
}

int64_t mctdh_profile_read(mctdh_ctx_t* ctx, int64_t kid, double* ms, int64_t* launches, double* flops,
                           double* bytes) {
  if (!ctx || kid < 0 || kid >= KP_N) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    drain_profile(*c);
    const KProf& k = c->prof[kid];
    if (ms) *ms = k.ms;
    if (launches) *launches = k.launches;
    if (flops) *flops = k.flops;
    if (bytes) *bytes = k.bytes;
  });
}

int64_t mctdh_observables(mctdh_ctx_t* ctx, double t, double* energy, double* pop, double* norm,
                          double* auto_re, double* auto_im) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  (void)t;
  return guarded(c, [&] { observables(*c, energy, pop, norm, auto_re, auto_im); });
}

int64_t mctdh_expect(mctdh_ctx_t* ctx, double* values) {
  if (!ctx) return MCTDH_EARG;
  Ctx* c = ctx->c;
  if (c->nexpect > 0 && !values) return MCTDH_EARG;
  return guarded(c, [&] {
    if (c->nexpect > 0) expectation(*c, (cplx*)values);
  });
}

int64_t mctdh_natpop(mctdh_ctx_t* ctx, double* nat, double* ggp, double* poperr) {
  if (!ctx || !nat) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] { natpop(*c, nat, ggp, poperr); });
}

int64_t mctdh_density(mctdh_ctx_t* ctx, int64_t dof, const double* trafo, int64_t ldt, double xmin, double xmax,
                      double* dens, double* pop) {
  if (!ctx || !dens) return MCTDH_EARG;
  Ctx* c = ctx->c;
  if (dof < 0 || dof >= c->ndof) return MCTDH_EARG;
  return guarded(c, [&] { density(*c, (int)dof, trafo, (int)ldt, xmin, xmax, dens, pop); });
}

int64_t mctdh_densmat(mctdh_ctx_t* ctx, int64_t mode, int64_t state, double* rho) {
  if (!ctx || !rho) return MCTDH_EARG;
  Ctx* c = ctx->c;
  if (mode < 0 || mode >= c->nmodes || state < 0 || state >= c->nstates) return MCTDH_EARG;
  return guarded(c, [&] {
    operators_and_mf(*c, c->d_y);
    const int n = c->m_of((int)mode, (int)state);
    CK(cudaMemcpyAsync(rho, c->rho[mode][state], sizeof(cplx) * n * n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    check_status(*c);
  });
}

int64_t mctdh_norm_wf(mctdh_ctx_t* ctx, const double* A, const double* psi, double* norm) {
  if (!ctx || !A || !psi || !norm) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_in, A, psi);
    upload(*c, c->d_out, A, psi);
    run_ovl(*c, c->io_plan);
    cplx o[3];
    read_ovl(*c, c->io_plan, o);
    *norm = o[0].x;
  });
}

int64_t mctdh_device_bytes(mctdh_ctx_t* ctx, int64_t* bytes) {
  if (!ctx || !bytes) return MCTDH_EARG;
  *bytes = (int64_t)ctx->c->ar.total;
  return MCTDH_OK;
}

int64_t mctdh_packets(mctdh_ctx_t* ctx, double* wppop, double* entropy) {
  if (!ctx || !wppop) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    copy_dev(*c, c->d_in, c->d_y, c->ntot);
    copy_dev(*c, c->d_out, c->d_y, c->ntot);
    run_ovl(*c, c->io_plan);
    std::vector<cplx> v(3 * c->npk);
    CK(cudaMemcpyAsync(v.data(), c->io_plan.d_result, sizeof(cplx) * v.size(), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    std::vector<double> w(c->npk);
    double tot = 0.0;
    for (int i = 0; i < c->npk; ++i) tot += (w[i] = v[3 * i].x);
    double ent = 0.0;
    for (int i = 0; i < c->npk; ++i) {
      w[i] /= tot;
      if (w[i] >= 1e-8) ent -= w[i] * log(w[i]);
    }
    std::sort(w.begin(), w.end(), [](double a, double b) { return a > b; });
    for (int i = 0; i < c->npk; ++i) wppop[i] = w[i];
    if (entropy) *entropy = c->npk > 1 ? ent / log((double)c->npk) : 0.0;
  });
}

int64_t mctdh_wf_ovl(mctdh_ctx_t* ctx, const double* A1, const double* psi1, const double* A2,
                     const double* psi2, double* re, double* im) {
  if (!ctx || !A1 || !psi1 || !A2 || !psi2 || !re || !im) return MCTDH_EARG;
  Ctx* c = ctx->c;
  return guarded(c, [&] {
    upload(*c, c->d_in, A1, psi1);
    upload(*c, c->d_out, A2, psi2);
    run_ovl(*c, c->io_plan);
    cplx o[3];
    read_ovl(*c, c->io_plan, o);
    *re = o[2].x;
    *im = o[2].y;
  });
}


// ---------------------------------------------------------------------------
// Ensembles
// ---------------------------------------------------------------------------
int64_t mctdh_ens_create(const mctdh_setup_t* setups, int64_t n, mctdh_ens_t** out) {
  if (!setups || !out || n < 1) return MCTDH_EARG;
  *out = nullptr;
  try {
    Ens* e = ens_create(setups, (int)n);
    if (tc_enabled()) tc_prepare();
    *out = new mctdh_ens{e};
    g_create_error.clear();
    return MCTDH_OK;
  } catch (const StatusError& e) {
    g_create_error = e.what();
    return e.code;
  } catch (const CudaError& e) {
    g_create_error = e.what();
    return MCTDH_ECUDA;
  } catch (const std::exception& e) {
    g_create_error = e.what();
    return MCTDH_EARG;
  }
}

int64_t mctdh_ens_destroy(mctdh_ens_t* ens) {
  if (!ens) return MCTDH_EARG;
  ens_destroy(ens->e);
  delete ens;
  return MCTDH_OK;
}

int64_t mctdh_ens_set_state(mctdh_ens_t* ens, int64_t i, const double* A, const double* psi, int64_t as_start) {
  if (!ens || !A || !psi || i < 0 || i >= (int64_t)ens->e->m.size()) return MCTDH_EARG;
  return ens_guarded(ens, [&] {
    Ctx& c = *ens->e->m[i];
    upload(c, c.d_y, A, psi);
    if (as_start) copy_dev(c, c.d_y0, c.d_y, c.ntot);
    CK(cudaStreamSynchronize(c.st));
  });
}

int64_t mctdh_ens_get_state(mctdh_ens_t* ens, int64_t i, double* A, double* psi) {
  if (!ens || !A || !psi || i < 0 || i >= (int64_t)ens->e->m.size()) return MCTDH_EARG;
  return ens_guarded(ens, [&] {
    Ctx& c = *ens->e->m[i];
    download(c, c.d_y, A, psi);
  });
}

int64_t mctdh_ens_calc_derivs(mctdh_ens_t* ens) {
  if (!ens) return MCTDH_EARG;
  return ens_guarded(ens, [&] {
    Ens& E = *ens->e;
    CK(cudaMemcpyAsync(E.IN, E.Y, sizeof(cplx) * E.total, cudaMemcpyDeviceToDevice, E.st));
    ens_eom(E, E.OUT);
    ens_check_status(E);
  });
}

int64_t mctdh_ens_get_derivs(mctdh_ens_t* ens, int64_t i, double* dA, double* dpsi) {
  if (!ens || !dA || !dpsi || i < 0 || i >= (int64_t)ens->e->m.size()) return MCTDH_EARG;
  return ens_guarded(ens, [&] {
    Ctx& c = *ens->e->m[i];
    download(c, c.d_out, dA, dpsi);
  });
}

int64_t mctdh_ens_propagate(mctdh_ens_t* ens, int64_t int_type, double tnext, double* t, double* step,
                            int64_t* nrounds, int64_t* neom) {
  if (!ens || !t || !step) return MCTDH_EARG;
  if (int_type != 1 && int_type != 2) return MCTDH_EUNSUPPORTED;
  return ens_guarded(ens, [&] {
    Ens& E = *ens->e;
    const long long r0 = E.rounds, e0 = E.eom_count;
    ens_propagate(E, (int)int_type, tnext, t, step);
    if (nrounds) *nrounds = E.rounds - r0;
    if (neom) *neom = E.eom_count - e0;
  });
}

int64_t mctdh_ens_observables(mctdh_ens_t* ens, int64_t i, double* energy, double* pop, double* norm,
                              double* auto_re, double* auto_im) {
  if (!ens || i < 0 || i >= (int64_t)ens->e->m.size()) return MCTDH_EARG;
  return ens_guarded(ens, [&] { observables(*ens->e->m[i], energy, pop, norm, auto_re, auto_im); });
}

int64_t mctdh_ens_counters(mctdh_ens_t* ens, int64_t* launches, int64_t* eom, int64_t* rounds) {
  if (!ens) return MCTDH_EARG;
  if (launches) *launches = ens->e->launches;
  if (eom) *eom = ens->e->eom_count;
  if (rounds) *rounds = ens->e->rounds;
  return MCTDH_OK;
}

int64_t mctdh_ens_autotune(mctdh_ens_t* ens, int64_t mode) {
  if (!ens || mode < 0 || mode > 2) return MCTDH_EARG;
  Ens& E = *ens->e;
  if (E.graph[0] || E.graph[1] || E.graph[2])
    return MCTDH_EARG;   // the launch shapes are fixed once a propagation captured its graphs
  try {
    if (mode == 0 || mode == 2) {
      E.tuned = true;    // keep the planned shapes
      if (mode == 2) {
        // persistent kernels on a minimal grid (4 mode-product and 2 contraction
        // CTAs), so that every CTA walks many blocks: the check that the
        // persistent forms repeat the per-block arithmetic
        E.persist_prod = 4;
        E.persist_hole = 2;
      }
      return MCTDH_OK;
    }
    E.tuned = false;
    ens_autotune(E);
    return MCTDH_OK;
  } catch (const StatusError& e) {
    E.last_error = e.what();
    return e.code;
  } catch (const std::exception& e) {
    E.last_error = e.what();
    return MCTDH_ECUDA;
  }
}

int64_t mctdh_ens_tuning(mctdh_ens_t* ens, int64_t* tiles_per_block, int64_t* block_cap, int64_t* tensor_cores,
                         double* eom_ms, double* default_eom_ms, int64_t* candidates) {
  if (!ens) return MCTDH_EARG;
  const Ens& E = *ens->e;
  if (tiles_per_block) *tiles_per_block = E.tune_tpb;
  if (block_cap) *block_cap = E.tune_cap;
  if (tensor_cores) *tensor_cores = (E.tune_tc && E.precision == 1 && tc_enabled()) ? 1 : 0;
  if (eom_ms) *eom_ms = E.tune_ms;
  if (default_eom_ms) *default_eom_ms = E.tune_default_ms;
  if (candidates) *candidates = E.tune_candidates;
  return MCTDH_OK;
}

int64_t mctdh_ens_persistent(mctdh_ens_t* ens, int64_t* prod_ctas, int64_t* hole_ctas) {
  if (!ens) return MCTDH_EARG;
  if (prod_ctas) *prod_ctas = ens->e->persist_prod;
  if (hole_ctas) *hole_ctas = ens->e->persist_hole;
  return MCTDH_OK;
}

int64_t mctdh_ens_eom_cost(mctdh_ens_t* ens, double* flops, double* bytes) {
  if (!ens) return MCTDH_EARG;
  const Ens& E = *ens->e;
  double fl = 0.0, by = 0.0;
  for (const auto* v : {&E.chains, &E.chains_full})
    for (const ProdBatch& b : *v) {
      fl += b.flops;
      by += b.bytes;
    }
  fl += E.gprods.flops;
  by += E.gprods.bytes;
  for (const HoleBatch* hb : {&E.rho_holes, &E.holes}) {
    fl += hb->flops;
    by += hb->bytes;
  }
  if (flops) *flops = fl;
  if (bytes) *bytes = by;
  return MCTDH_OK;
}

int64_t mctdh_ens_stream(mctdh_ens_t* ens, void** stream) {
  if (!ens || !stream) return MCTDH_EARG;
  *stream = (void*)ens->e->st;
  return MCTDH_OK;
}

const char* mctdh_ens_last_error(mctdh_ens_t* ens) {
  if (!ens) return g_create_error.c_str();
  return ens->e->last_error.c_str();
}

}  // extern "C"
