// grx_server.cu -- continuous-batching job server for Widom and GCMC jobs.
//
// Jobs (a box plus its work) are queued by grx_server_submit. grx_server_progress,
// called in the caller's loop, does one non-blocking scheduling round:
//   retire  jobs whose last slice finished: reduce the results, destroy the box
//           (its memory returns to the arena without a device-wide wait);
//   admit   queued jobs in arrival order while a slot is free and the job's box fits
//           in the arena (admission by HBM footprint);
//   launch  the next slice of every resident job without a slice in flight, each job
//           on its own non-blocking stream, so slices of different jobs overlap.
// A job's arithmetic is independent of the other resident jobs: it sees only its own
// box, and its Philox stream is fixed by its own seed, so its result is the same alone
// and in any mix.
//
// With gcmc_batching, GCMC jobs are not launched one by one: every round advances all
// resident GCMC jobs in one persistent launch of 8 warps per job (three jobs per SM, the
// shape of the batched benchmark), each job drawing from its own move stream and taking a
// number of steps set by its estimated cost per step, so that the jobs of a round end at
// about the same time. Jobs are admitted and retired between rounds; the round's batch is
// rebuilt when its membership changes. Widom jobs keep their own launches and streams.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <deque>
#include <mutex>
#include <vector>

#include "grx_host.h"

namespace grx {

struct ServerJob {
  uint64_t id = 0, tag = 0;
  int32_t kind = GRX_JOB_WIDOM;
  // owned copies of the inputs
  grx_box_desc desc{};
  std::vector<double> eps, sig, z, shift, c10;
  std::vector<std::vector<double>> pos, scale, charge, scc;
  std::vector<std::vector<size_t>> type, molid;
  std::vector<size_t> size, n_stored;
  std::vector<int32_t> rigid;
  grx_widom_desc widom{};
  int64_t total = 0;  // insertions or steps
  std::vector<grx_gcmc_desc> gcmc;
  // resident state
  grx_box* box = nullptr;
  grx_gcmc_batch* batch = nullptr;
  grx_widom_result* d_results = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  bool inflight = false;
  int64_t issued = 0;
  size_t footprint = 0;
  double t_submit = 0, t_admit = 0, t_done = 0;
  grx_status status = GRX_OK;
  // batched GCMC rounds
  std::vector<grx_gcmc_stats> acc;  // statistics summed over the rounds, one per move set
  int64_t tick_n = 0;               // steps of the round in flight
  bool in_tick = false;
  double cost = 1.0;                // estimated pair evaluations per step
};

}  // namespace grx

using namespace grx;

struct grx_server {
  grx_server_config cfg{};
  grx_arena* arena = nullptr;
  bool own_arena = false;
  std::deque<ServerJob*> pending;
  std::vector<ServerJob*> resident;
  std::vector<grx_job_result> done;
  std::vector<cudaStream_t> streams;  // idle streams for reuse
  std::chrono::steady_clock::time_point t0;
  uint64_t next_id = 1;
  uint64_t launches = 0;
  std::mutex m;
  // batched GCMC rounds (cfg.gcmc_batching)
  grx_gcmc_batch* tick = nullptr;
  std::vector<ServerJob*> tick_jobs;  // the batch's boxes, in order
  bool tick_inflight = false;
  cudaEvent_t tick_ev = nullptr;
  cudaStream_t tick_stream = nullptr;
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

grx_status release_job(grx_server* S, ServerJob* j) {
  if (j->batch) grx_gcmc_batch_destroy(j->batch);
  j->batch = nullptr;
  if (j->d_results) arena_free(S->arena, j->d_results);
  j->d_results = nullptr;
  if (j->box) grx_box_destroy(j->box);
  j->box = nullptr;
  if (j->ev) cudaEventDestroy(j->ev);
  j->ev = nullptr;
  if (j->stream) S->streams.push_back(j->stream);
  j->stream = nullptr;
  return GRX_OK;
}

// Creates the job's box in the arena and uploads its state. GRX_ERR_OUT_OF_MEMORY
// means "does not fit now" (nothing is left allocated).
grx_status admit_job(grx_server* S, ServerJob* j) {
  size_t before = 0;
  grx_arena_usage(S->arena, &before, nullptr, nullptr);
  grx_status st = grx_box_create_in(&j->desc, S->arena, &j->box);
  if (st) return st;
  // server boxes keep the tile path: voxel candidate lists would take arena memory only when
  // room allows, and a job's arithmetic must not depend on what else is resident
  j->box->vox_mode = 0;
  if (!S->streams.empty()) {
    j->stream = S->streams.back();
    S->streams.pop_back();
  } else {
    GRX_CHECK_CUDA(cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking), "job stream");
  }
  GRX_CHECK_CUDA(cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming), "job event");
  for (int c = 0; c < j->desc.ncomponents && st == GRX_OK; ++c) {
    grx_atoms a{};
    a.pos = j->pos[c].data();
    a.scale = j->scale[c].data();
    a.charge = j->charge[c].data();
    a.scale_coul = j->scc[c].data();
    a.type = j->type[c].data();
    a.molid = j->molid[c].data();
    a.size = j->size[c];
    a.n_stored = j->n_stored[c];
    st = grx_box_set_component(j->box, c, &a, j->rigid[c]);
  }
  if (st == GRX_OK) {
    double out8[8];
    st = grx_ewald_total(j->box, out8);
  }
  if (st == GRX_OK) st = grx_box_set_stream(j->box, j->stream);
  if (st == GRX_OK && j->kind == GRX_JOB_GCMC && S->cfg.gcmc_batching) {
    // cost per step in pair evaluations: the moved molecule's beads against the framework
    // atoms within the cutoff (at most all of them) and the guests, plus the Fourier
    // delta's k-vector updates of a charged molecule (weighted as 0.2 pair each)
    const grx_box* b = j->box;
    const int nh = (int)b->off[b->nhost];
    const double rc = std::sqrt(std::max(b->dev.cut_vdw2, b->dev.no_charges ? 0.0 : b->dev.cut_coul2));
    const double near = std::min((double)nh, 1.5 * nh / std::fabs(b->dev.volume) * 4.18879 * rc * rc * rc);
    double c = 0.0;
    for (const grx_gcmc_desc& d : j->gcmc) {
      const double ms = (double)b->molsize[d.component];
      c += ms * (near + 20.0);
      if (!b->dev.no_charges && b->has_charge[d.component]) c += 0.2 * b->nact * ms;
    }
    j->cost = std::max(1.0, c / (double)j->gcmc.size());
    j->acc.assign(j->gcmc.size(), grx_gcmc_stats{});
  } else if (st == GRX_OK && j->kind == GRX_JOB_GCMC) {
    const int32_t nm = (int32_t)j->gcmc.size();
    st = grx_gcmc_batch_create(&j->box, 1, j->gcmc.data(), &nm, S->cfg.precision, &j->batch);
    if (st == GRX_OK && S->cfg.cluster_atoms > 0) {  // a large box spans several SMs
      int64_t natoms = 0;
      for (int c = 0; c < j->desc.ncomponents; ++c) natoms += (int64_t)j->size[c];
      for (int32_t cl : {8, 4, 2}) {
        if (natoms < cl * S->cfg.cluster_atoms) continue;
        if (grx_gcmc_batch_set_shape(j->batch, 24, 1) == GRX_OK && grx_gcmc_batch_set_cluster(j->batch, cl) == GRX_OK)
          break;
      }
    }
  }
  if (st == GRX_OK && j->kind == GRX_JOB_WIDOM) {
    j->d_results = (grx_widom_result*)arena_alloc(S->arena, std::max<int64_t>(j->total, 1) * sizeof(grx_widom_result));
    if (!j->d_results) st = GRX_ERR_OUT_OF_MEMORY;
  }
  if (st) {
    release_job(S, j);
    if (st == GRX_ERR_OUT_OF_MEMORY) cudaGetLastError();
    return st;
  }
  size_t after = 0;
  grx_arena_usage(S->arena, &after, nullptr, nullptr);
  j->footprint = after - before;
  return GRX_OK;
}

grx_status launch_slice(grx_server* S, ServerJob* j) {
  const int64_t left = j->total - j->issued;
  grx_status st = GRX_OK;
  if (j->kind == GRX_JOB_WIDOM) {
    const int64_t n = std::min<int64_t>(left, std::max<int64_t>(S->cfg.widom_slice, 1));
    st = grx_widom_insertions_async(j->box, &j->widom, (uint64_t)j->issued, (size_t)n, S->cfg.precision,
                                    j->d_results + j->issued);
    j->issued += n;
  } else {
    const int64_t n = std::min<int64_t>(left, std::max<int64_t>(S->cfg.gcmc_slice, 1));
    st = grx_gcmc_batch_launch(j->batch, n, j->stream);
    j->issued += n;
  }
  if (st) return st;
  GRX_CHECK_CUDA(cudaEventRecord(j->ev, j->stream), "job event");
  j->inflight = true;
  S->launches++;
  return GRX_OK;
}

grx_status collect(grx_server* S, ServerJob* j, grx_job_result& r) {
  r = grx_job_result{};
  r.tag = j->tag;
  r.job_id = j->id;
  r.kind = j->kind;
  r.status = j->status;
  r.t_submit = j->t_submit;
  r.t_admit = j->t_admit;
  r.footprint_bytes = j->footprint;
  if (j->status == GRX_OK && j->kind == GRX_JOB_WIDOM) {
    std::vector<grx_widom_result> h((size_t)j->total);
    if (j->total)
      GRX_CHECK_CUDA(cudaMemcpyAsync(h.data(), j->d_results, j->total * sizeof(grx_widom_result),
                                     cudaMemcpyDeviceToHost, j->stream),
                     "widom results");
    GRX_CHECK_CUDA(cudaStreamSynchronize(j->stream), "widom results");
    double s = 0.0, s2 = 0.0;
    const bool chain = j->box && j->box->molsize[j->widom.component] > 1;
    int64_t cfg = 0;
    for (const grx_widom_result& x : h) {
      const double w = x.success ? x.rosenbluth : 0.0;
      s += w;
      s2 += w * w;
      cfg += j->widom.ntrials + (chain && x.w_first > 0.0 ? j->widom.norient : 0);
    }
    r.widom_trial_configs = cfg;
    r.widom_n = j->total;
    r.widom_mean_w = j->total ? s / (double)j->total : 0.0;
    r.widom_mean_w2 = j->total ? s2 / (double)j->total : 0.0;
  } else if (j->status == GRX_OK) {
    std::vector<grx_gcmc_stats> st(j->gcmc.size());
    if (j->batch) {
      grx_status e = grx_gcmc_batch_stats(j->batch, st.data(), nullptr);
      if (e) return e;
    } else {
      st = j->acc;
    }
    r.ncomp_moved = (int32_t)st.size();
    for (size_t k = 0; k < st.size() && k < 4; ++k) r.gcmc[k] = st[k];
    r.gcmc_steps = j->total;
  }
  r.t_done = S->now();
  return GRX_OK;
}

void add_stats(grx_gcmc_stats& a, const grx_gcmc_stats& b) {
  for (int k = 0; k < 5; ++k) {
    a.attempts[k] += b.attempts[k];
    a.accepted[k] += b.accepted[k];
  }
  a.n_molecules = b.n_molecules;
  a.capacity_hits += b.capacity_hits;
  for (int k = 0; k < 4; ++k) a.energy[k] += b.energy[k];
  a.sum_n += b.sum_n;
  for (int k = 0; k < 2; ++k) {
    a.identity_out[k] += b.identity_out[k];
    a.identity_in[k] += b.identity_in[k];
  }
  for (int k = 0; k < 3; ++k) a.rosen[k] += b.rosen[k];
  a.trial_configs += b.trial_configs;
  a.trial_beads += b.trial_beads;
}

// Ends the GCMC round in flight once its event completed: each member's statistics and steps.
grx_status finish_tick(grx_server* S) {
  if (!S->tick_inflight) return GRX_OK;
  const cudaError_t e = cudaEventQuery(S->tick_ev);
  if (e == cudaErrorNotReady) return GRX_OK;
  S->tick_inflight = false;
  grx_status st = e == cudaSuccess ? GRX_OK : cuda_status(e, "gcmc round");
  std::vector<grx_gcmc_stats> v;
  if (!st) {
    size_t ne = 0;
    for (ServerJob* j : S->tick_jobs) ne += j->gcmc.size();
    v.resize(ne);
    st = grx_gcmc_batch_stats(S->tick, v.data(), nullptr);
    if (!st) st = grx_gcmc_batch_reset_stats(S->tick);
  }
  size_t e0 = 0;
  for (ServerJob* j : S->tick_jobs) {
    if (st) j->status = st;
    else
      for (size_t k = 0; k < j->gcmc.size(); ++k) add_stats(j->acc[k], v[e0 + k]);
    e0 += j->gcmc.size();
    if (j->in_tick) {
      j->issued += j->tick_n;
      j->tick_n = 0;
      j->in_tick = false;
    }
  }
  return GRX_OK;
}

// Starts the next GCMC round over every resident GCMC job with steps left (the batch is
// rebuilt when the members changed). A job of estimated cost c pair evaluations per step
// takes gcmc_slice * 1000 / c steps, so the members of a round end at about the same time.
grx_status start_tick(grx_server* S) {
  if (S->tick_inflight) return GRX_OK;
  std::vector<ServerJob*> members;
  for (ServerJob* j : S->resident)
    if (j->kind == GRX_JOB_GCMC && j->status == GRX_OK && j->issued < j->total) members.push_back(j);
  if (members.empty()) return GRX_OK;
  if (!S->tick || members != S->tick_jobs) {
    if (S->tick) grx_gcmc_batch_destroy(S->tick);
    S->tick = nullptr;
    S->tick_jobs.clear();
    std::vector<grx_box*> boxes;
    std::vector<grx_gcmc_desc> descs;
    std::vector<int32_t> nm;
    for (ServerJob* j : members) {
      boxes.push_back(j->box);
      descs.insert(descs.end(), j->gcmc.begin(), j->gcmc.end());
      nm.push_back((int32_t)j->gcmc.size());
    }
    grx_status st = grx_gcmc_batch_create(boxes.data(), (int32_t)boxes.size(), descs.data(), nm.data(),
                                          S->cfg.precision, &S->tick);
    if (st == GRX_ERR_OUT_OF_MEMORY) {  // no room for the round's descriptors now: the next round retries
      cudaGetLastError();
      S->tick = nullptr;
      return GRX_OK;
    }
    if (st) return st;
    // one shape for every round (the same arithmetic alone and in any mix)
    st = grx_gcmc_batch_set_shape(S->tick, 8, 1);
    if (st) return st;
    for (ServerJob* j : members) GRX_CHECK_CUDA(cudaStreamSynchronize(j->stream), "gcmc round set-up");
    S->tick_jobs = members;
  }
  std::vector<uint64_t> next(members.size());
  std::vector<int64_t> n(members.size());
  int64_t nmax = 0;
  for (size_t i = 0; i < members.size(); ++i) {
    ServerJob* j = members[i];
    const double want = (double)S->cfg.gcmc_slice * 1000.0 / j->cost;
    n[i] = std::max<int64_t>(1, std::min<int64_t>(j->total - j->issued, (int64_t)std::llround(want)));
    next[i] = (uint64_t)j->issued;
    nmax = std::max(nmax, n[i]);
  }
  grx_status st = grx_gcmc_batch_set_box_steps(S->tick, next.data(), n.data());
  if (st) return st;
  st = grx_gcmc_batch_launch(S->tick, nmax, S->tick_stream);
  if (st) return st;
  GRX_CHECK_CUDA(cudaEventRecord(S->tick_ev, S->tick_stream), "gcmc round event");
  for (size_t i = 0; i < members.size(); ++i) {
    members[i]->tick_n = n[i];
    members[i]->in_tick = true;
  }
  S->tick_inflight = true;
  S->launches++;
  return GRX_OK;
}

}  // namespace

extern "C" grx_status grx_server_create(const grx_server_config* cfg, grx_arena* arena, grx_server** out) {
  GRX_REQUIRE(cfg && out, "grx_server_create: null argument");
  GRX_REQUIRE(cfg->max_resident >= 1, "grx_server_create: max_resident must be >= 1");
  GRX_REQUIRE(cfg->precision == GRX_FP64 || cfg->precision == GRX_MIXED || cfg->precision == GRX_FP32,
              "grx_server_create: bad precision");
  auto* S = new grx_server();
  S->cfg = *cfg;
  if (S->cfg.widom_slice <= 0) S->cfg.widom_slice = 1 << 30;
  if (S->cfg.gcmc_slice <= 0) S->cfg.gcmc_slice = 1 << 30;
  if (arena) {
    S->arena = arena;
  } else {
    grx_status st = grx_arena_create(cfg->hbm_budget_bytes, &S->arena);
    if (st) {
      delete S;
      return st;
    }
    S->own_arena = true;
  }
  if (S->cfg.gcmc_batching) {
    if (cudaStreamCreateWithFlags(&S->tick_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&S->tick_ev, cudaEventDisableTiming) != cudaSuccess) {
      const cudaError_t e = cudaGetLastError();
      if (S->tick_stream) cudaStreamDestroy(S->tick_stream);
      if (S->own_arena) grx_arena_destroy(S->arena);
      delete S;
      return cuda_status(e, "grx_server_create: round stream");
    }
  }
  S->t0 = std::chrono::steady_clock::now();
  *out = S;
  return GRX_OK;
}

extern "C" grx_status grx_server_destroy(grx_server* S) {
  if (!S) return GRX_OK;
  if (S->tick_stream) cudaStreamSynchronize(S->tick_stream);
  if (S->tick) grx_gcmc_batch_destroy(S->tick);
  S->tick = nullptr;
  for (ServerJob* j : S->resident) {
    if (j->stream) cudaStreamSynchronize(j->stream);
    release_job(S, j);
    delete j;
  }
  for (ServerJob* j : S->pending) delete j;
  for (cudaStream_t s : S->streams) cudaStreamDestroy(s);
  if (S->tick_ev) cudaEventDestroy(S->tick_ev);
  if (S->tick_stream) cudaStreamDestroy(S->tick_stream);
  if (S->own_arena) grx_arena_destroy(S->arena);
  delete S;
  return GRX_OK;
}

extern "C" grx_status grx_server_submit(grx_server* S, const grx_job_desc* jd, uint64_t* job_id) {
  GRX_REQUIRE(S && jd && jd->box && jd->atoms, "grx_server_submit: null argument");
  GRX_REQUIRE(jd->kind == GRX_JOB_WIDOM || jd->kind == GRX_JOB_GCMC, "grx_server_submit: bad job kind");
  const grx_box_desc& d = *jd->box;
  GRX_REQUIRE(d.ncomponents >= 1 && d.ncomponents <= GRX_MAX_COMPONENTS, "grx_server_submit: bad components");
  auto* j = new ServerJob();
  j->kind = jd->kind;
  j->tag = jd->tag;
  j->desc = d;
  const grx_forcefield& ff = d.forcefield;
  const size_t nt2 = (size_t)ff.ntypes * ff.ntypes;
  auto cp = [&](const double* p, std::vector<double>& v) {
    if (p) v.assign(p, p + nt2);
  };
  cp(ff.epsilon, j->eps);
  cp(ff.sigma, j->sig);
  cp(ff.z, j->z);
  cp(ff.shift, j->shift);
  cp(ff.c10, j->c10);
  j->desc.forcefield.epsilon = j->eps.empty() ? nullptr : j->eps.data();
  j->desc.forcefield.sigma = j->sig.empty() ? nullptr : j->sig.data();
  j->desc.forcefield.z = j->z.empty() ? nullptr : j->z.data();
  j->desc.forcefield.shift = j->shift.empty() ? nullptr : j->shift.data();
  j->desc.forcefield.c10 = j->c10.empty() ? nullptr : j->c10.data();
  const int nc = d.ncomponents;
  j->pos.resize(nc); j->scale.resize(nc); j->charge.resize(nc); j->scc.resize(nc);
  j->type.resize(nc); j->molid.resize(nc); j->size.resize(nc); j->n_stored.resize(nc); j->rigid.resize(nc);
  for (int c = 0; c < nc; ++c) {
    const grx_atoms& a = jd->atoms[c];
    const size_t n = std::max(a.size, a.n_stored);
    j->size[c] = a.size;
    j->n_stored[c] = n;
    j->pos[c].assign(a.pos, a.pos + 3 * n);
    j->charge[c].assign(a.charge, a.charge + n);
    j->type[c].assign(a.type, a.type + n);
    j->molid[c].assign(a.molid, a.molid + n);
    j->scale[c] = a.scale ? std::vector<double>(a.scale, a.scale + n) : std::vector<double>(n, 1.0);
    j->scc[c] = a.scale_coul ? std::vector<double>(a.scale_coul, a.scale_coul + n) : std::vector<double>(n, 1.0);
    j->rigid[c] = jd->rigid ? jd->rigid[c] : (c >= d.nhost_components ? 1 : 0);
  }
  if (jd->kind == GRX_JOB_WIDOM) {
    GRX_REQUIRE(jd->widom_insertions >= 0, "grx_server_submit: negative insertion count");
    j->widom = jd->widom;
    j->total = jd->widom_insertions;
  } else {
    GRX_REQUIRE(jd->gcmc && jd->ncomp_moved >= 1 && jd->ncomp_moved <= 4 && jd->gcmc_steps >= 0,
                "grx_server_submit: GCMC job needs 1..4 move sets and a step count");
    j->gcmc.assign(jd->gcmc, jd->gcmc + jd->ncomp_moved);
    j->total = jd->gcmc_steps;
  }
  std::lock_guard<std::mutex> g(S->m);
  j->id = S->next_id++;
  j->t_submit = S->now();
  S->pending.push_back(j);
  if (job_id) *job_id = j->id;
  return GRX_OK;
}

extern "C" grx_status grx_server_progress(grx_server* S, int32_t* n_resident, int32_t* n_pending) {
  GRX_REQUIRE(S, "grx_server_progress: null server");
  std::lock_guard<std::mutex> g(S->m);
  if (S->cfg.gcmc_batching) {
    grx_status st = finish_tick(S);
    if (st) return st;
  }
  // retire / advance resident jobs
  for (size_t i = 0; i < S->resident.size();) {
    ServerJob* j = S->resident[i];
    if (j->kind == GRX_JOB_GCMC && S->cfg.gcmc_batching) {  // advanced by the rounds
      if (j->in_tick || (j->status == GRX_OK && j->issued < j->total)) { ++i; continue; }
    } else if (j->inflight) {
      const cudaError_t e = cudaEventQuery(j->ev);
      if (e == cudaErrorNotReady) { ++i; continue; }
      j->inflight = false;
      if (e != cudaSuccess) j->status = cuda_status(e, "job slice");
    }
    if (j->status == GRX_OK && j->issued < j->total && !(j->kind == GRX_JOB_GCMC && S->cfg.gcmc_batching)) {
      j->status = launch_slice(S, j);
      if (j->status == GRX_OK) { ++i; continue; }
    }
    grx_job_result r;
    grx_status st = collect(S, j, r);
    if (st && r.status == GRX_OK) r.status = st;
    if (std::find(S->tick_jobs.begin(), S->tick_jobs.end(), j) != S->tick_jobs.end()) {
      // the (idle) round batch holds this job's box: drop it before the box goes
      grx_gcmc_batch_destroy(S->tick);
      S->tick = nullptr;
      S->tick_jobs.clear();
    }
    release_job(S, j);
    S->done.push_back(r);
    delete j;
    S->resident.erase(S->resident.begin() + i);
  }
  // admit in arrival order while slots and memory allow
  while (!S->pending.empty() && (int)S->resident.size() < S->cfg.max_resident) {
    ServerJob* j = S->pending.front();
    const grx_status st = admit_job(S, j);
    if (st == GRX_ERR_OUT_OF_MEMORY && !S->resident.empty()) break;  // wait for memory to free up
    S->pending.pop_front();
    if (st) {  // does not fit even alone, or invalid: report and drop
      j->status = st;
      grx_job_result r{};
      r.tag = j->tag;
      r.job_id = j->id;
      r.kind = j->kind;
      r.status = st;
      r.t_submit = j->t_submit;
      r.t_done = S->now();
      S->done.push_back(r);
      delete j;
      continue;
    }
    j->t_admit = S->now();
    S->resident.push_back(j);
    if (!(j->kind == GRX_JOB_GCMC && S->cfg.gcmc_batching)) j->status = j->total > 0 ? launch_slice(S, j) : GRX_OK;
  }
  if (S->cfg.gcmc_batching) {
    grx_status st = start_tick(S);
    if (st) return st;
  }
  if (n_resident) *n_resident = (int32_t)S->resident.size();
  if (n_pending) *n_pending = (int32_t)S->pending.size();
  return GRX_OK;
}

extern "C" grx_status grx_server_poll(grx_server* S, grx_job_result* out, int32_t max, int32_t* n) {
  GRX_REQUIRE(S && n && (out || max == 0), "grx_server_poll: bad argument");
  std::lock_guard<std::mutex> g(S->m);
  const int32_t k = std::min<int32_t>(max, (int32_t)S->done.size());
  for (int32_t i = 0; i < k; ++i) out[i] = S->done[i];
  S->done.erase(S->done.begin(), S->done.begin() + k);
  *n = k;
  return GRX_OK;
}

extern "C" grx_status grx_server_time(grx_server* S, double* seconds) {
  GRX_REQUIRE(S && seconds, "grx_server_time: bad argument");
  *seconds = S->now();
  return GRX_OK;
}

extern "C" grx_status grx_server_launch_count(grx_server* S, uint64_t* launches) {
  GRX_REQUIRE(S && launches, "grx_server_launch_count: bad argument");
  *launches = S->launches;
  return GRX_OK;
}
