// Serving loop: continuous batching of complete NRG runs.
//
// Requests (a whole run: models, hoppings, tracked operators, FDM spectrum
// and thermodynamics) arrive from any host thread through nrg_server_submit
// and wait in a FIFO queue.  Each worker thread owns one engine (its own
// CUDA stream) and repeats a tick:
//   1. admit queued requests while its active count is below max_active and
//      below its even share of all active and queued runs, and while their
//      estimated device footprint fits the HBM budget next to the
//      reservations of every active run (an idle server admits one request
//      regardless, so a request larger than the budget still runs alone);
//   2. advance every active run in its forward phase by one Wilson site:
//      one nrg_batch_add_site / nrg_opset_update_batch /
//      nrg_batch_update_state per hopping count, so the blocks of runs at
//      different sites share every launch, with the snapshot of each run in
//      between (update_system_operator and saveCurrentData, in the
//      reference's order);
//   3. run the backward passes (FDM spectrum, thermodynamics) of the runs
//      that finished their last site, shell by shell from the last, the FDM
//      shells of all of them in one nrg_fdm_calc_batch per step; collect
//      their results and free them.
// Requests that arrive while a tick is on the GPU join at the next tick.
// While one worker's host thread prepares its next launches, the kernels of
// the other workers' ticks keep the GPU busy.
// The footprint estimate is coef * nsites * (bath states * nkeep)^2 bytes;
// coef starts at 2 and is raised to 1.1x the largest ratio a finished run
// has shown (its peak device bytes over the same product).
//
// The worker calls only the public C ABI (include/nrg_gpu.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "nrg_gpu.h"

namespace nrg {
extern thread_local std::string g_err;  // nrg_last_error() text of this thread
}

namespace {

using Clock = std::chrono::steady_clock;

double seconds(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

struct ServeError {
  int code;
  std::string msg;
};

// Owned deep copy of an nrg_site_desc.
struct SiteCopy {
  std::vector<int> qnum, dims, blk_op, blk_row, blk_col;
  std::vector<double> energies, chi, blk_data;
  nrg_site_desc desc{};
  int64_t states = 0;
  void copy(const nrg_site_desc *d, bool need_chi) {
    if (!d || d->nq <= 0 || d->nsect <= 0 || !d->qnum || !d->dims || !d->energies)
      throw ServeError{NRG_E_ARG, "request: incomplete site description"};
    if (need_chi && !d->chi) throw ServeError{NRG_E_ARG, "request: bath site needs chi"};
    qnum.assign(d->qnum, d->qnum + int64_t(d->nq) * d->nsect);
    dims.assign(d->dims, d->dims + d->nsect);
    for (int x : dims) {
      if (x < 0) throw ServeError{NRG_E_ARG, "request: negative sector dimension"};
      states += x;
    }
    energies.assign(d->energies, d->energies + states);
    if (d->chi) chi.assign(d->chi, d->chi + d->nsect);
    if (d->nblk < 0 || (d->nblk > 0 && (!d->blk_op || !d->blk_row || !d->blk_col || !d->blk_data)))
      throw ServeError{NRG_E_ARG, "request: operator blocks missing"};
    blk_op.assign(d->blk_op, d->blk_op + d->nblk);
    blk_row.assign(d->blk_row, d->blk_row + d->nblk);
    blk_col.assign(d->blk_col, d->blk_col + d->nblk);
    int64_t nd = 0;
    for (int b = 0; b < d->nblk; ++b) {
      if (blk_row[b] < 0 || blk_row[b] >= d->nsect || blk_col[b] < 0 || blk_col[b] >= d->nsect)
        throw ServeError{NRG_E_ARG, "request: operator block sector out of range"};
      nd += int64_t(dims[blk_row[b]]) * dims[blk_col[b]];
    }
    blk_data.assign(d->blk_data, d->blk_data + nd);
    desc = *d;
    desc.qnum = qnum.data();
    desc.dims = dims.data();
    desc.energies = energies.data();
    desc.chi = chi.empty() ? nullptr : chi.data();
    desc.blk_op = blk_op.data();
    desc.blk_row = blk_row.data();
    desc.blk_col = blk_col.data();
    desc.blk_data = blk_data.data();
  }
};

// Owned deep copy of an nrg_op_desc.
struct OpsCopy {
  std::vector<int> op, row, col, rows, cols;
  std::vector<double> data;
  nrg_op_desc desc{};
  void copy(const nrg_op_desc *d) {
    if (d->nblk < 0 || (d->nblk > 0 && (!d->blk_op || !d->blk_row || !d->blk_col || !d->blk_rows ||
                                        !d->blk_cols || !d->blk_data)))
      throw ServeError{NRG_E_ARG, "request: tracked operator blocks missing"};
    op.assign(d->blk_op, d->blk_op + d->nblk);
    row.assign(d->blk_row, d->blk_row + d->nblk);
    col.assign(d->blk_col, d->blk_col + d->nblk);
    rows.assign(d->blk_rows, d->blk_rows + d->nblk);
    cols.assign(d->blk_cols, d->blk_cols + d->nblk);
    int64_t nd = 0;
    for (int b = 0; b < d->nblk; ++b) {
      if (rows[b] < 0 || cols[b] < 0) throw ServeError{NRG_E_ARG, "request: negative operator block size"};
      nd += int64_t(rows[b]) * cols[b];
    }
    data.assign(d->blk_data, d->blk_data + nd);
    desc = *d;
    desc.blk_op = op.data();
    desc.blk_row = row.data();
    desc.blk_col = col.data();
    desc.blk_rows = rows.data();
    desc.blk_cols = cols.data();
    desc.blk_data = data.data();
  }
};

constexpr int kFdmPoints = 100000;

struct Job {
  uint64_t id = 0;
  // request
  SiteCopy imp, bath;
  uint64_t nkeep = 0;
  int nsites = 0, nt = 0;
  std::vector<double> t, rescale, shell_scale, temps;
  bool has_ops = false, fdm = false, keep_eigs = false;
  OpsCopy ops;
  int first_shell_site = 0;
  double estimate = 0;  // reserved device bytes
  // state
  nrg_run *run = nullptr;
  nrg_opset *opset = nullptr;
  int site = 0;
  struct Shell {
    int64_t iteration;
    int site;
  };
  std::vector<Shell> shells;
  int64_t peak_bytes = 0;
  // results
  bool done = false;
  int status = NRG_OK;
  std::string message;
  std::vector<double> eigs;
  std::vector<uint64_t> eig_counts;
  std::vector<double> energy_points, positive, negative, entropy, cv;
  Clock::time_point t_submit, t_admit, t_finish;
  bool admitted = false;  // counted in the server's active runs and reservation

  void release_device() {
    if (opset) nrg_opset_destroy(opset);
    opset = nullptr;
    if (run) nrg_run_destroy(run);
    run = nullptr;
  }
};

void check(int rc, const char *what) {
  if (rc != NRG_OK) throw ServeError{rc, std::string(what) + ": " + nrg_last_error()};
}

}  // namespace

struct Worker {
  nrg_engine *eng = nullptr;
  bool owns_engine = false;
  std::thread th;
  std::vector<std::shared_ptr<Job>> active;  // touched by this worker's thread only
};

struct nrg_server {
  int device = 0;  // CUDA device current when the server was created
  int max_active = 16;
  uint64_t budget = 0;
  double coef = 2.0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<std::shared_ptr<Job>> queue;
  std::map<uint64_t, std::shared_ptr<Job>> jobs;  // every job not yet released
  std::vector<std::unique_ptr<Worker>> workers;
  uint64_t n_active = 0;  // admitted, not finished (all workers)
  double reserved = 0;    // footprint estimates of those runs
  uint64_t next_id = 1;
  bool stop = false;
  // statistics
  uint64_t submitted = 0, completed = 0, failed = 0, max_active_seen = 0, ticks = 0;
  double busy_s = 0;
  std::vector<double> latencies;

  double estimate(const Job &j) const {
    const double s = double(j.bath.states) * double(j.nkeep);
    return coef * double(j.nsites) * s * s;
  }
  void loop(Worker &w);
  void tick(std::vector<std::shared_ptr<Job>> &act);
  void backward(std::vector<Job *> &fin);
  void finish(Job &j, int status, const std::string &msg);
};

void nrg_server::finish(Job &j, int status, const std::string &msg) {
  j.release_device();
  std::lock_guard<std::mutex> lk(mu);
  if (j.admitted) {
    j.admitted = false;
    --n_active;
    reserved -= j.estimate;
    cv_work.notify_all();  // budget and a share slot freed: waiting workers may admit
  }
  j.status = status;
  j.message = msg;
  j.t_finish = Clock::now();
  j.done = true;
  if (status == NRG_OK) {
    ++completed;
    latencies.push_back(seconds(j.t_submit, j.t_finish));
    const double s = double(j.bath.states) * double(j.nkeep);
    const double ratio = double(j.peak_bytes) / std::max(1.0, double(j.nsites) * s * s);
    coef = std::max(coef, 1.1 * ratio);
  } else {
    ++failed;
  }
  cv_done.notify_all();
}

void nrg_server::loop(Worker &w) {
  cudaSetDevice(device);  // the runtime's current device is per host thread
  std::vector<std::shared_ptr<Job>> &active = w.active;
  const uint64_t nworkers = workers.size();
  for (;;) {
    std::vector<std::shared_ptr<Job>> admitted;
    {
      std::unique_lock<std::mutex> lk(mu);
      if (stop) break;
      if (active.empty() && queue.empty()) {
        cv_work.wait_for(lk, std::chrono::milliseconds(50));
        continue;
      }
      // even share of the active and queued runs over the workers
      const uint64_t share = (n_active + queue.size() + nworkers - 1) / nworkers;
      const uint64_t cap = std::min<uint64_t>(uint64_t(max_active), std::max<uint64_t>(share, 1));
      while (!queue.empty() && active.size() + admitted.size() < cap) {
        auto &q = queue.front();
        const double est = estimate(*q);
        const bool idle = n_active == 0;
        if (budget && !idle && reserved + est > double(budget)) break;
        q->estimate = est;
        q->t_admit = Clock::now();
        q->admitted = true;
        reserved += est;
        ++n_active;
        admitted.push_back(q);
        queue.pop_front();
      }
      max_active_seen = std::max<uint64_t>(max_active_seen, n_active);
      if (active.empty() && admitted.empty()) {
        // queued work this worker may not take yet (the budget is held by
        // other workers' runs): wait for a finish or a submission
        cv_work.wait_for(lk, std::chrono::milliseconds(50));
        continue;
      }
    }
    for (auto &j : admitted) {
      try {
        check(nrg_run_create(w.eng, &j->imp.desc, &j->bath.desc, j->nkeep, &j->run), "run create");
        active.push_back(j);
      } catch (const ServeError &x) {
        finish(*j, x.code, x.msg);
      }
    }
    if (active.empty()) continue;
    const auto t0 = Clock::now();
    tick(active);
    const auto t1 = Clock::now();
    std::lock_guard<std::mutex> lk(mu);
    busy_s += seconds(t0, t1);
    ++ticks;
  }
  // stopped: fail what this worker still runs; the queue is failed by the
  // server once every worker has stopped
  for (auto &j : active)
    if (!j->done) finish(*j, NRG_E_STATE, "server stopped");
}

static void fail_queue(nrg_server *s) {
  std::vector<std::shared_ptr<Job>> rest;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    rest.assign(s->queue.begin(), s->queue.end());
    s->queue.clear();
  }
  for (auto &j : rest) s->finish(*j, NRG_E_STATE, "server stopped");
}

void nrg_server::tick(std::vector<std::shared_ptr<Job>> &act) {
  // ---- forward: one site for every active run, batched per hopping count
  std::map<int, std::vector<Job *>> groups;
  for (auto &j : act) groups[j->nt].push_back(j.get());
  for (auto &g : groups) {
    std::vector<Job *> &js = g.second;
    const int nt = g.first;
    std::vector<nrg_run *> runs;
    std::vector<double> t, rs;
    for (Job *j : js) {
      runs.push_back(j->run);
      t.insert(t.end(), j->t.begin() + int64_t(j->site) * nt, j->t.begin() + int64_t(j->site + 1) * nt);
      rs.push_back(j->rescale[j->site]);
    }
    int rc = nrg_batch_add_site(runs.data(), int(runs.size()), t.data(), nt, rs.data());
    if (rc != NRG_OK) {  // isolate the failing run(s): step each run alone
      const std::string msg = nrg_last_error();
      std::vector<Job *> ok;
      for (Job *j : js) {
        int r1 = nrg_run_add_site(j->run, j->t.data() + int64_t(j->site) * nt, nt, j->rescale[j->site]);
        if (r1 == NRG_OK) ok.push_back(j);
        else finish(*j, r1, std::string("add_site: ") + nrg_last_error());
      }
      (void)msg;
      js = ok;
      runs.clear();
      for (Job *j : js) runs.push_back(j->run);
    }
    // tracked operators of all runs of the group in one batched update
    std::vector<Job *> with_ops;
    for (Job *j : js) {
      try {
        if (j->has_ops && j->site == 0) check(nrg_opset_create(j->run, &j->ops.desc, &j->opset), "opset");
        if (j->opset) with_ops.push_back(j);
      } catch (const ServeError &x) {
        finish(*j, x.code, x.msg);
      }
    }
    if (!with_ops.empty()) {
      std::vector<nrg_opset *> os;
      for (Job *j : with_ops) os.push_back(j->opset);
      if (nrg_opset_update_batch(os.data(), int(os.size())) != NRG_OK) {
        for (Job *j : with_ops) {  // isolate the failing run(s)
          const int r1 = nrg_opset_update(j->opset);
          if (r1 != NRG_OK) finish(*j, r1, std::string("opset update: ") + nrg_last_error());
        }
      }
    }
    std::vector<Job *> stepped;
    for (Job *j : js) {
      if (j->done) continue;
      try {
        if ((j->fdm || !j->temps.empty()) && j->site >= j->first_shell_site) {
          int disc = 0;
          check(nrg_run_check_discarded(j->run, &disc), "check discarded");
          if (disc) {
            nrg_run_info info{};
            check(nrg_run_get_info(j->run, &info), "info");
            check(nrg_run_snapshot(j->run, j->opset), "snapshot");
            j->shells.push_back({info.iteration, j->site});
          }
        }
        stepped.push_back(j);
      } catch (const ServeError &x) {
        finish(*j, x.code, x.msg);
      }
    }
    std::vector<nrg_run *> sr;
    for (Job *j : stepped) sr.push_back(j->run);
    if (!sr.empty()) {
      rc = nrg_batch_update_state(sr.data(), int(sr.size()));
      if (rc != NRG_OK) {
        for (Job *j : stepped) {
          int r1 = nrg_run_update_state(j->run);
          if (r1 != NRG_OK) finish(*j, r1, std::string("update_state: ") + nrg_last_error());
        }
      }
    }
    for (Job *j : stepped) {
      if (j->done) continue;
      try {
        nrg_run_info info{};
        check(nrg_run_get_info(j->run, &info), "info");
        j->peak_bytes = std::max<int64_t>(j->peak_bytes, info.device_bytes);
        if (j->keep_eigs) {
          const size_t o = j->eigs.size();
          j->eigs.resize(o + size_t(info.n_all));
          check(nrg_run_get_all_eigenvalues(j->run, j->eigs.data() + o, uint64_t(info.n_all)), "eigenvalues");
          j->eig_counts.push_back(uint64_t(info.n_all));
        }
        ++j->site;
      } catch (const ServeError &x) {
        finish(*j, x.code, x.msg);
      }
    }
  }
  // ---- backward passes of the runs that finished their last site
  std::vector<Job *> fin;
  for (auto &jp : act)
    if (!jp->done && jp->site >= jp->nsites) fin.push_back(jp.get());
  if (!fin.empty()) backward(fin);
  act.erase(std::remove_if(act.begin(), act.end(), [](const std::shared_ptr<Job> &j) { return j->done; }),
            act.end());
}

// Backward passes of the runs in `fin`, shell by shell from each run's last
// shell: step r loads the r-th last snapshot of every run that has one and
// bins the FDM shells of all of them in one nrg_fdm_calc_batch (a run's
// shells stay in the reference's order; the runs only share launches).
void nrg_server::backward(std::vector<Job *> &fin) {
  struct Pass {
    Job *j;
    nrg_fdm *f = nullptr;
    nrg_thermo *th = nullptr;
  };
  std::vector<Pass> ps;
  for (Job *j : fin) {
    Pass p{j};
    try {
      const int nops = j->has_ops ? j->ops.desc.nops : 0;
      if (j->fdm) check(nrg_fdm_create(j->run, nops, &p.f), "fdm create");
      if (!j->temps.empty())
        check(nrg_thermo_create(j->run, j->temps.data(), int(j->temps.size()), &p.th), "thermo create");
      ps.push_back(p);
    } catch (const ServeError &x) {
      if (p.f) nrg_fdm_destroy(p.f);
      if (p.th) nrg_thermo_destroy(p.th);
      finish(*j, x.code, x.msg);
    }
  }
  auto fail = [&](Pass &p, const ServeError &x) {
    if (p.f) nrg_fdm_destroy(p.f);
    if (p.th) nrg_thermo_destroy(p.th);
    p.f = nullptr;
    p.th = nullptr;
    finish(*p.j, x.code, x.msg);
  };
  size_t depth = 0;
  for (auto &p : ps) depth = std::max(depth, p.j->shells.size());
  for (size_t r = 0; r < depth; ++r) {
    std::vector<Pass *> step;
    for (auto &p : ps) {
      if (p.j->done || r >= p.j->shells.size()) continue;
      try {
        check(nrg_run_load_snapshot(p.j->run, p.j->shells[p.j->shells.size() - 1 - r].iteration), "load snapshot");
        step.push_back(&p);
      } catch (const ServeError &x) {
        fail(p, x);
      }
    }
    std::vector<nrg_fdm *> fs;
    std::vector<double> sc;
    for (Pass *p : step) {
      if (!p->f) continue;
      fs.push_back(p->f);
      sc.push_back(p->j->shell_scale[p->j->shells[p->j->shells.size() - 1 - r].site]);
    }
    if (!fs.empty() && nrg_fdm_calc_batch(fs.data(), int(fs.size()), sc.data()) != NRG_OK) {
      for (Pass *p : step) {  // isolate the failing run(s)
        if (!p->f) continue;
        const int r1 = nrg_fdm_calc(p->f, p->j->shell_scale[p->j->shells[p->j->shells.size() - 1 - r].site]);
        if (r1 != NRG_OK) fail(*p, ServeError{r1, std::string("fdm calc: ") + nrg_last_error()});
      }
    }
    for (Pass *p : step) {
      if (p->j->done || !p->th) continue;
      try {
        check(nrg_thermo_calc(p->th, p->j->shell_scale[p->j->shells[p->j->shells.size() - 1 - r].site]),
              "thermo calc");
      } catch (const ServeError &x) {
        fail(*p, x);
      }
    }
  }
  for (auto &p : ps) {
    Job &j = *p.j;
    if (j.done) continue;
    try {
      const int nops = j.has_ops ? j.ops.desc.nops : 0;
      if (p.f) {
        j.energy_points.assign(kFdmPoints, 0.0);
        j.positive.assign(size_t(nops) * kFdmPoints, 0.0);
        j.negative.assign(size_t(nops) * kFdmPoints, 0.0);
        check(nrg_fdm_get(p.f, j.energy_points.data(), j.positive.data(), j.negative.data(), kFdmPoints),
              "fdm get");
      }
      if (p.th) {
        j.entropy.assign(j.temps.size(), 0.0);
        j.cv.assign(j.temps.size(), 0.0);
        check(nrg_thermo_final(p.th, j.entropy.data(), j.cv.data()), "thermo final");
      }
      nrg_run_info info{};
      check(nrg_run_get_info(j.run, &info), "info");
      j.peak_bytes = std::max<int64_t>(j.peak_bytes, info.device_bytes);
      if (p.f) nrg_fdm_destroy(p.f);
      if (p.th) nrg_thermo_destroy(p.th);
      p.f = nullptr;
      p.th = nullptr;
      finish(j, NRG_OK, "");
    } catch (const ServeError &x) {
      fail(p, x);
    }
  }
}

namespace {
template <class F> int sguard(F &&f) {
  try {
    f();
    return NRG_OK;
  } catch (const ServeError &e) {
    nrg::g_err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    nrg::g_err = e.what();
    return NRG_E_ARG;
  }
}

std::shared_ptr<Job> find_job(nrg_server *s, uint64_t id) {
  auto it = s->jobs.find(id);
  if (it == s->jobs.end()) throw ServeError{NRG_E_ARG, "unknown request id"};
  return it->second;
}
}  // namespace

extern "C" {

int nrg_server_create(nrg_engine *eng, const nrg_server_opts *opts, nrg_server **out) {
  return sguard([&] {
    if (!eng || !out) throw ServeError{NRG_E_ARG, "null argument"};
    auto s = std::make_unique<nrg_server>();
    if (cudaGetDevice(&s->device) != cudaSuccess) throw ServeError{NRG_E_NOCUDA, "no current CUDA device"};
    int nworkers = 1;
    if (opts) {
      if (opts->max_active < 1) throw ServeError{NRG_E_ARG, "max_active must be >= 1"};
      if (opts->workers < 0 || opts->workers > 64) throw ServeError{NRG_E_ARG, "workers must be in [0, 64]"};
      s->max_active = opts->max_active;
      s->budget = opts->hbm_budget_bytes;
      nworkers = std::max(1, opts->workers);
    }
    nrg_engine_opts eo{};
    check(nrg_engine_get_opts(eng, &eo), "engine options");
    for (int k = 0; k < nworkers; ++k) {
      auto w = std::make_unique<Worker>();
      w->eng = eng;
      if (k > 0) {
        const int rc = nrg_engine_create(&eo, &w->eng);
        if (rc != NRG_OK) {
          const std::string msg = nrg_last_error();
          for (auto &o : s->workers)
            if (o->owns_engine) nrg_engine_destroy(o->eng);
          throw ServeError{rc, "worker engine: " + msg};
        }
        w->owns_engine = true;
      }
      s->workers.push_back(std::move(w));
    }
    nrg_server *raw = s.get();
    for (auto &w : s->workers) {
      Worker *wp = w.get();
      w->th = std::thread([raw, wp] { raw->loop(*wp); });
    }
    *out = s.release();
  });
}

int nrg_server_destroy(nrg_server *s) {
  return sguard([&] {
    if (!s) return;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &w : s->workers)
      if (w->th.joinable()) w->th.join();
    fail_queue(s);
    for (auto &w : s->workers)
      if (w->owns_engine) nrg_engine_destroy(w->eng);
    delete s;
  });
}

int nrg_server_submit(nrg_server *s, const nrg_request *r, uint64_t *id) {
  return sguard([&] {
    if (!s || !r || !id) throw ServeError{NRG_E_ARG, "null argument"};
    if (r->nsites <= 0 || r->nt <= 0 || !r->t || !r->rescale)
      throw ServeError{NRG_E_ARG, "request: nsites, nt, t and rescale are required"};
    if (r->nkeep == 0) throw ServeError{NRG_E_ARG, "request: nkeep must be > 0"};
    if (r->fdm && !r->ops) throw ServeError{NRG_E_ARG, "request: the FDM spectrum needs tracked operators"};
    if ((r->fdm || r->ntemps > 0) && !r->shell_scale)
      throw ServeError{NRG_E_ARG, "request: the backward passes need shell_scale"};
    if (r->ntemps < 0 || (r->ntemps > 0 && !r->temps)) throw ServeError{NRG_E_ARG, "request: temperatures"};
    auto j = std::make_shared<Job>();
    j->imp.copy(r->impurity, false);
    j->bath.copy(r->bath, true);
    j->nkeep = r->nkeep;
    j->nsites = r->nsites;
    j->nt = r->nt;
    j->t.assign(r->t, r->t + int64_t(r->nsites) * r->nt);
    j->rescale.assign(r->rescale, r->rescale + r->nsites);
    if (r->shell_scale) j->shell_scale.assign(r->shell_scale, r->shell_scale + r->nsites);
    if (r->ntemps > 0) j->temps.assign(r->temps, r->temps + r->ntemps);
    j->has_ops = r->ops != nullptr;
    if (j->has_ops) j->ops.copy(r->ops);
    j->fdm = r->fdm != 0;
    j->keep_eigs = r->keep_eigenvalues != 0;
    j->first_shell_site = std::max(0, r->first_shell_site);
    j->t_submit = Clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) throw ServeError{NRG_E_STATE, "server stopped"};
      j->id = s->next_id++;
      s->jobs[j->id] = j;
      s->queue.push_back(j);
      ++s->submitted;
      *id = j->id;
    }
    s->cv_work.notify_all();
  });
}

int nrg_server_wait(nrg_server *s, uint64_t id, double timeout_s, int *done) {
  return sguard([&] {
    if (!s || !done) throw ServeError{NRG_E_ARG, "null argument"};
    std::unique_lock<std::mutex> lk(s->mu);
    auto j = find_job(s, id);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                          std::chrono::duration<double>(std::max(0.0, timeout_s)));
    s->cv_done.wait_until(lk, until, [&] { return j->done; });
    *done = j->done ? 1 : 0;
  });
}

int nrg_server_result_info(nrg_server *s, uint64_t id, nrg_result_info *info) {
  return sguard([&] {
    if (!s || !info) throw ServeError{NRG_E_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    auto j = find_job(s, id);
    *info = nrg_result_info{};
    info->done = j->done ? 1 : 0;
    info->status = j->status;
    if (!j->done) return;
    info->latency_s = seconds(j->t_submit, j->t_finish);
    info->queue_s = j->t_admit.time_since_epoch().count() ? seconds(j->t_submit, j->t_admit) : 0.0;
    info->nsites = j->nsites;
    info->n_eig_total = int64_t(j->eigs.size());
    info->nops = j->fdm ? j->ops.desc.nops : 0;
    info->npts = j->fdm ? kFdmPoints : 0;
    info->ntemps = int(j->temps.size());
    info->peak_device_bytes = uint64_t(j->peak_bytes);
    std::snprintf(info->message, sizeof(info->message), "%s", j->message.c_str());
  });
}

int nrg_server_get_result(nrg_server *s, uint64_t id, double *eigs, uint64_t *eig_counts,
                          double *energy_points, double *positive, double *negative, double *entropy,
                          double *cv) {
  return sguard([&] {
    if (!s) throw ServeError{NRG_E_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    auto j = find_job(s, id);
    if (!j->done) throw ServeError{NRG_E_STATE, "request not finished"};
    if (j->status != NRG_OK) throw ServeError{j->status, "request failed: " + j->message};
    auto put = [](double *dst, const std::vector<double> &v) {
      if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(double));
    };
    put(eigs, j->eigs);
    if (eig_counts && !j->eig_counts.empty())
      std::memcpy(eig_counts, j->eig_counts.data(), j->eig_counts.size() * sizeof(uint64_t));
    put(energy_points, j->energy_points);
    put(positive, j->positive);
    put(negative, j->negative);
    put(entropy, j->entropy);
    put(cv, j->cv);
  });
}

int nrg_server_release(nrg_server *s, uint64_t id) {
  return sguard([&] {
    if (!s) throw ServeError{NRG_E_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    auto j = find_job(s, id);
    if (!j->done) throw ServeError{NRG_E_STATE, "request not finished"};
    s->jobs.erase(id);
  });
}

int nrg_server_stats(nrg_server *s, nrg_server_stats_t *st, int reset) {
  return sguard([&] {
    if (!s || !st) throw ServeError{NRG_E_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    *st = nrg_server_stats_t{};
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->failed = s->failed;
    st->queued = s->queue.size();
    st->max_active_seen = s->max_active_seen;
    st->ticks = s->ticks;
    st->busy_s = s->busy_s;
    st->footprint_coef = s->coef;
    std::vector<double> l = s->latencies;
    if (!l.empty()) {
      std::sort(l.begin(), l.end());
      auto pct = [&](double p) {  // nearest-rank percentile
        size_t k = size_t(std::ceil(p * double(l.size())));
        if (k < 1) k = 1;
        return l[std::min(l.size(), k) - 1];
      };
      st->p50_latency_s = pct(0.50);
      st->p99_latency_s = pct(0.99);
      double sum = 0;
      for (double x : l) sum += x;
      st->mean_latency_s = sum / double(l.size());
      st->max_latency_s = l.back();
    }
    if (reset) {
      s->latencies.clear();
      s->max_active_seen = 0;
      s->busy_s = 0;
      s->ticks = 0;
    }
  });
}

}  // extern "C"
