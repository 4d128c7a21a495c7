// Batched RI JK builds (many molecules of different sizes) on the tensor cores:
// the three GEMM phases of every molecule (half transform, J, K) each run as
// ONE grouped launch over all molecules' tiles, and the whole sequence --
// per-molecule slicing and diagonal kernels included -- is captured once into
// a CUDA graph that gb_batch_launch replays (the per-molecule kernels as
// parallel branches of the graph).
//
// Tile configuration per phase (chosen by the caller, e.g. the autotuner in
// pynof_gb300/batch.py):
//   0  orbitals on the 128-row side (A = C^T slices), N tile 128;
//   1, 2, 3  operands swapped, orbitals on the N side with N tile 32, 64, 128
//      (small nbf5 then wastes less of each tile).
// The K phase (a symmetric SYRK per orbital) always uses configuration 0.
// A phase whose outputs store along the tile rows' unit stride (configuration
// 3, and K) runs as one persistent launch (one CTA per SM) over the
// concatenated tile space of all molecules, in order through a tile counter;
// the others run one CTA per tile.
#include <cstring>
#include <new>
#include <vector>

#include "ozaki_tc.cuh"
#include "ri_kernels.cuh"
#include "slice.cuh"

using namespace gb;

struct gb_batch {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int nmol = 0;
};

namespace {

struct MolWs {
  SlicedDesc A, d, T;
  double *Tf, *dv;
};

template <class Cv>
void mol_layout(Cv& c, int N, int P, int Q, int S, MolWs* w) {
  SlicedDesc A = take_sliced(c, 1, P, N, S);
  auto* tf = c.template take<double>((size_t)P * N * Q);
  auto* dv = c.template take<double>((size_t)P * Q);
  SlicedDesc d = take_sliced(c, 1, P, Q, S);
  SlicedDesc T = take_sliced(c, P, N, Q, S);
  if (w) *w = MolWs{A, d, T, tf, dv};
}


// Prepared-b layout (must match gb_ri_prepare_mixed).
void prepared_views(const void* prep, int N, int Q, int S, SlicedDesc* bT, SlicedDesc* bJ) {
  Carve c(const_cast<void*>(prep), (size_t)-1);
  *bT = take_sliced(c, 1, N * Q, N, S);
  *bJ = take_sliced(c, 1, N * (N + 1) / 2, Q, S);  // the pairs m <= n (the prepared layout)
}

int bn_of(int code) { return code == 1 ? 32 : code == 2 ? 64 : 128; }

}  // namespace

extern "C" size_t gb_jkj_batch_workspace_mixed(int nmol, const int* nbf, const int* nbf5, const int* naux,
                                               int nslices) {
  SizeCarve c;
  for (int i = 0; i < nmol; ++i) mol_layout(c, nbf[i], nbf5[i], naux[i], nslices, nullptr);
  c.used += 3 * ozaki_group_table_bytes(nmol);
  return c.used;
}

extern "C" int gb_jkj_batch_create_mixed(int nmol, const double* const* C, const void* const* prep, const int* nbf,
                                         const int* nbf5, const int* naux, int nslices, double* const* J,
                                         double* const* K, const int* tiles, void* workspace, size_t workspace_bytes,
                                         void* stream, gb_batch** plan) {
  clear_error();
  GB_REQUIRE(nmol >= 1 && C && prep && nbf && nbf5 && naux && J && K && plan, GB_ERR_INVALID_ARG,
             "gb_jkj_batch_create_mixed: null argument");
  GB_REQUIRE(valid_split(nslices), GB_ERR_INVALID_ARG,
             "gb_jkj_batch_create_mixed: nslices=%d is neither 1..6 nor GB_SPLIT_TF32X3", nslices);
  const int tcfg = tiles ? tiles[0] : 0, jcfg = tiles ? tiles[1] : 0;
  GB_REQUIRE(tcfg >= 0 && tcfg <= 3 && jcfg >= 0 && jcfg <= 3, GB_ERR_INVALID_ARG,
             "gb_jkj_batch_create_mixed: tile configuration outside [0, 3]");
  for (int i = 0; i < nmol; ++i) {
    GB_REQUIRE(nbf[i] > 0 && nbf5[i] > 0 && nbf5[i] <= nbf[i] && naux[i] > 0 && C[i] && prep[i] && J[i] && K[i],
               GB_ERR_BAD_SHAPE, "gb_jkj_batch_create_mixed: molecule %d has bad sizes or null buffers", i);
  }
  GB_REQUIRE(workspace_bytes >= gb_jkj_batch_workspace_mixed(nmol, nbf, nbf5, naux, nslices), GB_ERR_WORKSPACE,
             "gb_jkj_batch_create_mixed: workspace too small");
  const int S = nslices;
  Carve wc(workspace, workspace_bytes);
  std::vector<MolWs> ws(nmol);
  for (int i = 0; i < nmol; ++i) mol_layout(wc, nbf[i], nbf5[i], naux[i], S, &ws[i]);
  void* tabT = wc.take<unsigned char>(ozaki_group_table_bytes(nmol));
  void* tabJ = wc.take<unsigned char>(ozaki_group_table_bytes(nmol));
  void* tabK = wc.take<unsigned char>(ozaki_group_table_bytes(nmol));

  std::vector<OzProblem> pt(nmol), pj(nmol), pk(nmol);
  long long tilesT = 0, tilesJ = 0, tilesK = 0;
  for (int i = 0; i < nmol; ++i) {
    const int N = nbf[i], P = nbf5[i], Q = naux[i];
    SlicedDesc bT, bJ;
    prepared_views(prep[i], N, Q, S, &bT, &bJ);
    const MolWs& w = ws[i];
    OzGemm g{};
    g.S = S; g.batch = 1; g.c_sb = 0; g.sym = SYM_NONE;
    if (tcfg == 0) {  // T[q][j] = sum_m C[m][q] b[m][j]
      g.M = P; g.N = N * Q; g.K = N; g.bn = 128;
      g.C = w.Tf; g.c_r = lin((long long)N * Q); g.c_c = lin(1);
      pt[i] = OzProblem{w.A, bT, g};
    } else {
      g.M = N * Q; g.N = P; g.K = N; g.bn = bn_of(tcfg);
      g.C = w.Tf; g.c_r = lin(1); g.c_c = lin((long long)N * Q);
      pt[i] = OzProblem{bT, w.A, g};
    }
    tilesT += ozaki_tiles(pt[i].g);
    OzGemm h{};
    h.S = S; h.batch = 1; h.c_sb = 0; h.pair_n = N; h.K = Q;
    if (jcfg == 0) {  // J[q][(m,n)] = sum_l d[q][l] b[(m,n)][l], pairs m <= n, mirrored
      h.M = P; h.N = N * (N + 1) / 2; h.bn = 128; h.sym = SYM_TRICOL;
      h.C = J[i]; h.c_r = lin((long long)N * N); h.c_c = lin(1);
      pj[i] = OzProblem{w.d, bJ, h};
    } else {
      h.M = N * (N + 1) / 2; h.N = P; h.bn = bn_of(jcfg); h.sym = SYM_TRIROW;
      h.C = J[i]; h.c_r = lin(1); h.c_c = lin((long long)N * N);
      pj[i] = OzProblem{bJ, w.d, h};
    }
    tilesJ += ozaki_tiles(pj[i].g);
    OzGemm k{};
    k.S = S; k.M = N; k.N = N; k.K = Q; k.batch = P; k.bn = 128; k.sym = SYM_ROWCOL;
    k.C = K[i]; k.c_sb = (long long)N * N; k.c_r = lin(1); k.c_c = lin(N);  // symmetric: stored transposed
    pk[i] = OzProblem{w.T, w.T, k};
    tilesK += ozaki_tiles(pk[i].g);
  }
  // phases whose outputs store rows along their unit stride (orbitals on the
  // 128-wide N tile, and K) run as persistent grouped launches
  bool persT = false, persJ = false, persK = false;
  GB_TRY(ozaki_group_upload(pt.data(), nmol, tabT, &persT));
  GB_TRY(ozaki_group_upload(pj.data(), nmol, tabJ, &persJ));
  GB_TRY(ozaki_group_upload(pk.data(), nmol, tabK, &persK));

  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The per-molecule kernels between the grouped GEMMs (slicing, the diagonal
  // contraction) are small; they are captured as parallel branches on
  // kBranches forked streams (molecule i on branch i % kBranches), so the
  // replay runs several molecules' kernels at once instead of one after another.
  constexpr int kBranches = 8;
  const int nbr = nmol < kBranches ? nmol : kBranches;
  cudaStream_t aux[kBranches] = {};
  cudaEvent_t ev[4 * (kBranches + 1)] = {};
  auto release = [&]() {
    for (cudaEvent_t& e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaStream_t& a : aux)
      if (a) cudaStreamDestroy(a);
  };
  for (int j = 0; j < nbr; ++j) {
    const cudaError_t e = cudaStreamCreateWithFlags(&aux[j], cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      release();
      return cuda_status(e, "gb_jkj_batch_create_mixed: branch streams");
    }
  }
  for (cudaEvent_t& e : ev) {
    const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if (r != cudaSuccess) {
      release();
      return cuda_status(r, "gb_jkj_batch_create_mixed: branch events");
    }
  }
  int phase = 0;
  // run per_mol(i, stream) for every molecule on the branches, between a fork
  // from and a join back into the capturing stream
  auto branches = [&](auto&& per_mol) -> int {
    cudaEvent_t* pe = ev + (phase++) * (kBranches + 1);
    GB_TRY(cuda_status(cudaEventRecord(pe[0], s), "batch fork"));
    for (int j = 0; j < nbr; ++j) GB_TRY(cuda_status(cudaStreamWaitEvent(aux[j], pe[0], 0), "batch fork"));
    for (int i = 0; i < nmol; ++i) GB_TRY(per_mol(i, aux[i % nbr]));
    for (int j = 0; j < nbr; ++j) {
      GB_TRY(cuda_status(cudaEventRecord(pe[1 + j], aux[j]), "batch join"));
      GB_TRY(cuda_status(cudaStreamWaitEvent(s, pe[1 + j], 0), "batch join"));
    }
    return GB_OK;
  };
  GB_TRY(cuda_status(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"));
  int st = GB_OK;
  auto body = [&]() -> int {
    GB_TRY(branches([&](int i, cudaStream_t b) {
      return slice_operand(SliceSrc{C[i], 0, lin(1), lin(nbf[i]), false}, ws[i].A, b);
    }));
    GB_TRY(ozaki_gemm_grouped(tabT, nmol, tilesT, S, pt[0].g.bn, s, "ozaki_tc:batch_half_transform", persT));
    GB_TRY(branches([&](int i, cudaStream_t b) {
      GB_TRY(launch_contract_diag(C[i], ws[i].Tf, ws[i].dv, nbf[i], nbf5[i], naux[i], b));
      return slice_operand(SliceSrc{ws[i].dv, 0, lin(naux[i]), lin(1), true}, ws[i].d, b);
    }));
    GB_TRY(ozaki_gemm_grouped(tabJ, nmol, tilesJ, S, pj[0].g.bn, s, "ozaki_tc:batch_J", persJ));
    GB_TRY(branches([&](int i, cudaStream_t b) {
      return slice_operand(SliceSrc{ws[i].Tf, (long long)nbf[i] * naux[i], lin(naux[i]), lin(1), true}, ws[i].T, b);
    }));
    GB_TRY(ozaki_gemm_grouped(tabK, nmol, tilesK, S, 128, s, "ozaki_tc:batch_K", persK));
    return GB_OK;
  };
  st = body();
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(s, &graph);
  release();
  if (st != GB_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  GB_TRY(cuda_status(ec, "cudaStreamEndCapture"));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_status(ei, "cudaGraphInstantiate");
  }
  gb_batch* b = new (std::nothrow) gb_batch;
  if (!b) {
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    set_error(GB_ERR_INVALID_ARG, "gb_jkj_batch_create_mixed: out of host memory");
    return GB_ERR_INVALID_ARG;
  }
  b->graph = graph;
  b->exec = exec;
  b->nmol = nmol;
  *plan = b;
  return GB_OK;
}

extern "C" int gb_batch_launch(gb_batch* plan, void* stream) {
  clear_error();
  GB_REQUIRE(plan && plan->exec, GB_ERR_INVALID_ARG, "gb_batch_launch: no plan");
  return cuda_status(cudaGraphLaunch(plan->exec, static_cast<cudaStream_t>(stream)), "cudaGraphLaunch");
}

extern "C" int gb_batch_destroy(gb_batch* plan) {
  clear_error();
  if (!plan) return GB_OK;
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->graph) cudaGraphDestroy(plan->graph);
  delete plan;
  return GB_OK;
}
