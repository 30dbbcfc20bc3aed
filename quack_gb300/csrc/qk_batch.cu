// qk_batch.cu -- many independent GW systems of uneven size in one call.
//
// Systems are independent (no exchange step), so the batch is spread over a pool of worker
// sub-contexts, each with its own CUDA stream and workspace, driven by one host thread each.
// Workers pull systems from a shared queue ordered by decreasing cost (nS^3), so the large
// systems start first and the small ones fill the gaps; the GPU runs the workers' kernels
// concurrently (the cooperative tridiagonalisation of a small system occupies only a few SMs).
// The tridiagonalisations, the dominant cost, do not run one system at a time: the workers hand
// their matrices to a grouped launch (qk_tri_service, k_eig.cu) that tridiagonalises all the
// workers' current matrices at once, a CTA group per matrix sized by its share of the work, each
// group with its own bounded barrier -- one persistent cooperative launch per round instead of a
// whole-GPU launch per system.  The grouped kernel's arithmetic does not depend on the group's
// size, so results do not depend on which matrices share a launch.
// A failing or non-converged system is recorded in its status word and does not stop the batch.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>
#include "qk_internal.cuh"

namespace {

struct Item {
  int idx;
  double cost;
};

int make_worker(qk_ctx* parent, qk_ctx** out) {
  qk_ctx* w = nullptr;
  const int rc = qk_init(parent->device, &w);
  if (rc != QK_OK) return rc;
  *out = w;
  return QK_OK;
}

}  // namespace

extern "C" int qk_gw_batch_L_dev(qk_ctx* ctx, const qk_gw_params* prm, int method, int nsys,
                                 const qk_sys_desc* desc, const double* d_L, const double* d_eHF,
                                 double* d_eGW, double* EcRPA, int* status, int* nSCF,
                                 int n_workers) {
  if (!ctx || !prm || !desc || nsys < 0 || (method != 0 && method != 1)) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (n_workers < 1) n_workers = 1;
  if (n_workers > 32) n_workers = 32;
  if (n_workers > nsys) n_workers = nsys > 0 ? nsys : 1;
  while ((int)ctx->workers.size() < n_workers) {
    qk_ctx* w = nullptr;
    const int rc = make_worker(ctx, &w);
    if (rc != QK_OK) return qk_fail(ctx, rc, "could not create batch worker context");
    ctx->workers.push_back(w);
  }
  // each worker's cooperative tridiagonalisation gets a share of the SMs; every worker stream
  // starts after the caller's default-stream work (the packed inputs)
  const int share = ctx->num_sms / n_workers > 16 ? ctx->num_sms / n_workers : 16;
  for (int wi = 0; wi < n_workers; ++wi) {
    qk_ctx* w = ctx->workers[wi];
    w->sytrd_max_ctas = share;
    // the caller's tuned launch parameters and learned QP model apply to every worker (the
    // model is only read: its inference writes the worker's own workspace)
    std::memcpy(w->tune, ctx->tune, sizeof(ctx->tune));
    w->newton_maxit = ctx->newton_maxit;
    w->mlp = ctx->mlp;
    QK_TRY(qk_order_after_default(w));
  }
  qk_tri_service* svc = qk_tri_service_new(ctx, n_workers);
  if (!svc) return qk_fail(ctx, QK_ERR_CUDA, "could not create the grouped tridiagonalisation");
  for (int wi = 0; wi < n_workers; ++wi) ctx->workers[wi]->tri_service = svc;
  std::vector<Item> order(nsys);
  for (int i = 0; i < nsys; ++i) {
    const double nS = (double)(desc[i].nO - desc[i].nC) * (desc[i].nOrb - desc[i].nO - desc[i].nR);
    order[i] = {i, nS * nS * nS + (double)desc[i].nOrb * desc[i].nOrb * nS * nS};
  }
  std::sort(order.begin(), order.end(), [](const Item& a, const Item& b) { return a.cost > b.cost; });
  std::atomic<int> next(0);
  std::mutex err_mu;
  std::string first_err;
  auto run = [&](int wi) {
    qk_ctx* w = ctx->workers[wi];
    cudaSetDevice(w->device);
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= nsys) break;
      const int i = order[k].idx;
      const qk_sys_desc& s = desc[i];
      const int N = s.nOrb;
      double* sig = nullptr;
      int st = qk_wst(w, W_BATCHIO, (size_t)3 * N + 4096, &sig);
      double ec = 0.0, gm = 0.0, conv = 0.0;
      int ns = 0;
      if (st == QK_OK) {
        w->err.clear();
        (void)cudaGetLastError();
        st = qk_status_reset(w);
        if (st == QK_OK) {
          const double* L = d_L + s.offset_L;
          const double* e = d_eHF + s.offset_e;
          double* eg = d_eGW + s.offset_e;
          if (method == 0)
            st = qk_g0w0_L(w, prm, N, s.nC, s.nO, s.nR, s.naux, L, e, eg, sig, sig + N, sig + 2 * N,
                           &ec, &gm);
          else
            st = qk_evgw_L(w, prm, N, s.nC, s.nO, s.nR, s.naux, L, e, eg, sig, sig + N, &ec, &gm,
                           &ns, &conv);
        }
        if (st == QK_OK || st == QK_ERR_NO_CONV) {
          const int s2 = qk_status_check(w, QKD_BARRIER_TIMEOUT | QKD_BAD_INDEX | QKD_MBAR_TIMEOUT);
          if (s2 != QK_OK) st = s2;
        }
      }
      if (st != QK_OK && st != QK_ERR_NO_CONV) {
        std::lock_guard<std::mutex> lk(err_mu);
        if (first_err.empty()) first_err = "system " + std::to_string(i) + ": " + w->err;
      }
      if (status) status[i] = st;
      if (EcRPA) EcRPA[i] = ec;
      if (nSCF) nSCF[i] = method == 1 ? ns : 1;
    }
    qk_tri_service_worker_done(svc);
    cudaStreamSynchronize(w->stream);
  };
  std::vector<std::thread> th;
  for (int wi = 1; wi < n_workers; ++wi) th.emplace_back(run, wi);
  run(0);
  for (auto& t : th) t.join();
  for (int wi = 0; wi < n_workers; ++wi) ctx->workers[wi]->tri_service = nullptr;
  qk_tri_service_free(svc);
  long long launches = 0;
  for (auto* w : ctx->workers) launches += w->launches;
  ctx->launches = launches;  // for diagnostics: the batch's own launch total
  int worst = QK_OK;
  if (status)
    for (int i = 0; i < nsys; ++i)
      if (status[i] != QK_OK && status[i] != QK_ERR_NO_CONV) worst = status[i];
  if (worst != QK_OK) ctx->err = first_err;
  return worst;
}
