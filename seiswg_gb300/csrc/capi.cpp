// capi.cpp -- the extern "C" boundary declared in include/seiswg.h.
#include "../../include/seiswg.h"

#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "batch.h"
#include "host.h"

struct seiswg_vfs {
  seiswg::Vfs map;
};

struct seiswg_config {
  seiswg::Config cfg;
};

struct seiswg_sim {
  seiswg::Sim* sim = nullptr;
  bool owned = false;
};

struct seiswg_batch {
  std::unique_ptr<seiswg::Batch> batch;
};

struct seiswg_solver {
  std::unique_ptr<seiswg::Solver> solver;
  seiswg_sim view;
};

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace seiswg {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace seiswg

namespace {

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <typename F>
int guarded(F&& f) {
  try {
    g_last_error.clear();
    f();
    return SEISWG_OK;
  } catch (const seiswg::WaitTimeout& e) {
    return fail(SEISWG_ETIMEOUT, e.what());
  } catch (const seiswg::NumericError& e) {
    return fail(SEISWG_ENUMERIC, e.what());
  } catch (const seiswg::CudaError& e) {
    return fail(SEISWG_ECUDA, e.what());
  } catch (const seiswg::Error& e) {
    std::string m = e.what();
    bool io = m.rfind("Cannot read", 0) == 0 || m.rfind("Cannot open", 0) == 0 ||
              m.rfind("Cannot create", 0) == 0 || m.rfind("Cannot write", 0) == 0 ||
              m.rfind("Cannot load", 0) == 0;
    return fail(io ? SEISWG_EIO : SEISWG_EINVAL, m);
  } catch (const std::logic_error& e) {  // invalid arguments and out-of-order calls
    return fail(SEISWG_EINVAL, e.what());
  } catch (const std::bad_alloc&) {
    return fail(SEISWG_EINTERNAL, "host out of memory");
  } catch (const std::exception& e) {
    return fail(SEISWG_EINTERNAL, e.what());
  }
}

bool state_field(const char* name, seiswg::StateField* f) {
  static const struct {
    const char* n;
    seiswg::StateField f;
  } tab[] = {{"vy", seiswg::StateField::VY},   {"sxy", seiswg::StateField::SXY}, {"szy", seiswg::StateField::SZY},
             {"vx", seiswg::StateField::VX},   {"vz", seiswg::StateField::VZ},   {"sxx", seiswg::StateField::SXX},
             {"szz", seiswg::StateField::SZZ}, {"sxz", seiswg::StateField::SXZ}, {"vyc", seiswg::StateField::VYC},
             {"ry", seiswg::StateField::VYC},  {"syx", seiswg::StateField::SYX}, {"syy", seiswg::StateField::SYY},
             {"syz", seiswg::StateField::SYZ}};
  if (!name) return false;
  for (const auto& t : tab)
    if (std::strcmp(t.n, name) == 0) { *f = t.f; return true; }
  return false;
}

seiswg::Sim& sim_of(seiswg_sim* s) {
  if (!s || !s->sim) throw std::invalid_argument("null simulation handle");
  return *s->sim;
}

}  // namespace

extern "C" {

const char* seiswg_last_error(void) { return g_last_error.c_str(); }
const char* seiswg_version(void) { return "seiswg-gb300 0.1 (sm_103a)"; }

// ---- VFS --------------------------------------------------------------------
seiswg_vfs* seiswg_vfs_new(void) { return new (std::nothrow) seiswg_vfs(); }
void seiswg_vfs_free(seiswg_vfs* v) { delete v; }

int seiswg_vfs_insert(seiswg_vfs* v, const char* key, const void* data, size_t len) {
  if (!v || !key || (len && !data)) return fail(SEISWG_EINVAL, "seiswg_vfs_insert: null argument");
  return guarded([&] {
    const uint8_t* p = static_cast<const uint8_t*>(data);
    v->map[key] = seiswg::Bytes(p, p + len);
  });
}

int seiswg_vfs_get(const seiswg_vfs* v, const char* key, const void** data, size_t* len) {
  if (!v || !key || !data || !len) return fail(SEISWG_EINVAL, "seiswg_vfs_get: null argument");
  auto it = v->map.find(key);
  if (it == v->map.end()) return fail(SEISWG_EIO, std::string("VFS entry not found: ") + key);
  *data = it->second.data();
  *len = it->second.size();
  g_last_error.clear();
  return SEISWG_OK;
}

size_t seiswg_vfs_size(const seiswg_vfs* v) { return v ? v->map.size() : 0; }

const char* seiswg_vfs_key(const seiswg_vfs* v, size_t index) {
  if (!v || index >= v->map.size()) return nullptr;
  auto it = v->map.begin();
  std::advance(it, long(index));
  return it->first.c_str();
}

// ---- config -----------------------------------------------------------------
int seiswg_config_load(const char* path, seiswg_config** out) {
  if (!path || !out) return fail(SEISWG_EINVAL, "seiswg_config_load: null argument");
  *out = nullptr;
  return guarded([&] {
    std::unique_ptr<seiswg_config> c(new seiswg_config());
    try {
      c->cfg = seiswg::config_load(path);
    } catch (const seiswg::Error& e) {
      std::string m = e.what();
      if (m.rfind("Cannot open", 0) == 0) throw;
      throw seiswg::Error(std::string("Failed to load ") + path + ": " + m);
    }
    *out = c.release();
  });
}

int seiswg_config_load_str(const char* text, const char* base_dir, seiswg_config** out) {
  if (!text || !out) return fail(SEISWG_EINVAL, "seiswg_config_load_str: null argument");
  *out = nullptr;
  return guarded([&] {
    std::unique_ptr<seiswg_config> c(new seiswg_config());
    c->cfg = seiswg::config_load_str(text, base_dir ? base_dir : "");
    *out = c.release();
  });
}

void seiswg_config_free(seiswg_config* c) { delete c; }

int seiswg_config_get(const seiswg_config* c, const char* key, char* buf, size_t buflen) {
  if (!c || !key || !buf || buflen == 0) return fail(SEISWG_EINVAL, "seiswg_config_get: null argument");
  return guarded([&] {
    const seiswg::Config& k = c->cfg;
    std::string s, name = key;
    auto b = [](bool v) { return std::string(v ? "yes" : "no"); };
    auto f = [](float v) { char t[64]; std::snprintf(t, sizeof t, "%.9g", double(v)); return std::string(t); };
    bool found = true;
    if (name == "workflow") s = k.workflow;
    else if (name == "solver.sh") s = b(k.sh);
    else if (name == "solver.psv") s = b(k.psv);
    else if (name == "solver.spin") s = b(k.spin);
    else if (name == "solver.nt") s = std::to_string(k.nt);
    else if (name == "solver.dt") s = f(k.dt);
    else if (name == "solver.abs_left") s = b(k.abs_left);
    else if (name == "solver.abs_right") s = b(k.abs_right);
    else if (name == "solver.abs_bottom") s = b(k.abs_bottom);
    else if (name == "solver.abs_top") s = b(k.abs_top);
    else if (name == "solver.abs_width") s = std::to_string(k.abs_width);
    else if (name == "solver.abs_alpha") s = f(k.abs_alpha);
    else if (name == "solver.threads_per_block") s = std::to_string(k.threads_per_block);
    else if (name == "solver.combine_sources") s = b(k.combine_sources);
    else if (name == "solver.save_snapshot") s = std::to_string(k.save_snapshot);
    else if (name == "solver.adj_interval") s = std::to_string(k.adj_interval);
    else if (name == "solver.smooth") s = f(k.smooth);
    else if (name == "path.output") s = k.output;
    else if (name == "path.output_traces") { found = k.has_output_traces; s = k.output_traces; }
    else if (name == "path.model_true") { found = k.has_model_true; s = k.model_true; }
    else if (name == "path.model_init") { found = k.has_model_init; s = k.model_init; }
    else if (name == "path.sources") s = k.sources;
    else if (name == "path.stations") s = k.stations;
    else if (name == "path.traces") { found = k.has_traces; s = k.traces; }
    else throw std::invalid_argument(std::string("unknown config key ") + key);
    if (!found) throw std::invalid_argument(std::string("config key not set: ") + key);
    if (s.size() + 1 > buflen) throw std::invalid_argument("buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
  });
}

// ---- solver -----------------------------------------------------------------
int seiswg_solver_new(const seiswg_config* c, const seiswg_vfs* vfs, seiswg_solver** out) {
  if (!c || !out) return fail(SEISWG_EINVAL, "seiswg_solver_new: null argument");
  *out = nullptr;
  return guarded([&] {
    static const seiswg::Vfs empty;
    std::unique_ptr<seiswg_solver> s(new seiswg_solver());
    s->solver.reset(new seiswg::Solver(c->cfg, vfs ? vfs->map : empty));
    s->view.sim = &s->solver->sim();
    s->view.owned = false;
    *out = s.release();
  });
}

int seiswg_solver_set_write_files(seiswg_solver* s, int on) {
  if (!s) return fail(SEISWG_EINVAL, "null solver");
  s->solver->set_write_files(on != 0);
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_solver_run_forward(seiswg_solver* s, seiswg_vfs* out) {
  if (!s) return fail(SEISWG_EINVAL, "null solver");
  return guarded([&] {
    seiswg::Vfs r = s->solver->run_forward();
    if (out)
      for (auto& kv : r) out->map[kv.first] = std::move(kv.second);
  });
}

int seiswg_solver_run_adjoint(seiswg_solver* s, const seiswg_vfs* vfs, seiswg_vfs* out) {
  if (!s) return fail(SEISWG_EINVAL, "null solver");
  return guarded([&] {
    static const seiswg::Vfs empty;
    seiswg::Vfs r = s->solver->run_adjoint(vfs ? vfs->map : empty);
    if (out)
      for (auto& kv : r) out->map[kv.first] = std::move(kv.second);
  });
}

int seiswg_solver_run_inversion(seiswg_solver* s, const seiswg_vfs* vfs, seiswg_vfs* out) {
  if (!s) return fail(SEISWG_EINVAL, "null solver");
  return guarded([&] {
    static const seiswg::Vfs empty;
    seiswg::Vfs r = s->solver->run_inversion(vfs ? vfs->map : empty);
    if (out)
      for (auto& kv : r) out->map[kv.first] = std::move(kv.second);
  });
}

int seiswg_solver_info(const seiswg_solver* s, int32_t* nx, int32_t* nz, float* dx, float* dz, int32_t* nsrc,
                       int32_t* nrec) {
  if (!s) return fail(SEISWG_EINVAL, "null solver");
  if (nx) *nx = s->solver->nx();
  if (nz) *nz = s->solver->nz();
  if (dx) *dx = s->solver->dx();
  if (dz) *dz = s->solver->dz();
  if (nsrc) *nsrc = s->solver->nsrc();
  if (nrec) *nrec = s->solver->nrec();
  g_last_error.clear();
  return SEISWG_OK;
}

double seiswg_solver_total_misfit(const seiswg_solver* s) { return s ? s->solver->total_misfit() : 0.0; }

seiswg_sim* seiswg_solver_sim(seiswg_solver* s) { return s ? &s->view : nullptr; }

void seiswg_solver_free(seiswg_solver* s) { delete s; }

// ---- simulation operator ------------------------------------------------------
int seiswg_sim_create(const seiswg_sim_desc* d, void* stream, seiswg_sim** out) {
  if (!d || !out) return fail(SEISWG_EINVAL, "seiswg_sim_create: null argument");
  *out = nullptr;
  return guarded([&] {
    seiswg::SimDesc sd;
    sd.nx = d->nx; sd.nz = d->nz; sd.nt = d->nt;
    sd.dx = d->dx; sd.dz = d->dz; sd.dt = d->dt;
    sd.sh = d->sh != 0; sd.psv = d->psv != 0; sd.spin = d->spin != 0;
    sd.abs_left = d->abs_left != 0; sd.abs_right = d->abs_right != 0;
    sd.abs_bottom = d->abs_bottom != 0; sd.abs_top = d->abs_top != 0;
    sd.abs_width = d->abs_width; sd.abs_alpha = d->abs_alpha;
    std::unique_ptr<seiswg_sim> s(new seiswg_sim());
    s->sim = new seiswg::Sim(sd, static_cast<cudaStream_t>(stream));
    s->owned = true;
    *out = s.release();
  });
}

void seiswg_sim_free(seiswg_sim* s) {
  if (!s) return;
  if (s->owned) {
    delete s->sim;
    delete s;
  }
}

int seiswg_sim_upload_model(seiswg_sim* s, const char* name, const float* host, size_t n) {
  return guarded([&] {
    seiswg::Sim& sim = sim_of(s);
    if (!name || !host) throw std::invalid_argument("null model argument");
    if (n != size_t(sim.desc().nx) * size_t(sim.desc().nz))
      throw std::invalid_argument("model field size does not match nx*nz");
    static const struct {
      const char* n;
      seiswg::ModelField f;
    } tab[] = {{"vp", seiswg::ModelField::VP},       {"vs", seiswg::ModelField::VS},
               {"rho", seiswg::ModelField::RHO},     {"lambda", seiswg::ModelField::LAMBDA},
               {"mu", seiswg::ModelField::MU},       {"nu", seiswg::ModelField::NU},
               {"j", seiswg::ModelField::J},         {"lambda_c", seiswg::ModelField::LAMBDA_C},
               {"mu_c", seiswg::ModelField::MU_C},   {"nu_c", seiswg::ModelField::NU_C}};
    for (const auto& t : tab)
      if (std::strcmp(t.n, name) == 0) {
        sim.upload_model(t.f, host);
        return;
      }
    throw std::invalid_argument(std::string("unknown model field ") + name);
  });
}

int seiswg_sim_prepare(seiswg_sim* s) {
  return guarded([&] { sim_of(s).prepare_model(); });
}

int seiswg_sim_stability(const seiswg_sim* s, double* wave, double* spin) {
  if (!s || !s->sim) return fail(SEISWG_EINVAL, "null simulation handle");
  if (wave) *wave = s->sim->stability_wave();
  if (spin) *spin = s->sim->stability_spin();
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_sim_set_sources(seiswg_sim* s, int32_t n, const int32_t* i, const int32_t* j, const float* stf) {
  return guarded([&] {
    if (n > 0 && (!i || !j || !stf)) throw std::invalid_argument("null source argument");
    sim_of(s).set_sources(n, i, j, stf);
  });
}

int seiswg_sim_set_receivers(seiswg_sim* s, int32_t n, const int32_t* i, const int32_t* j) {
  return guarded([&] {
    if (n > 0 && (!i || !j)) throw std::invalid_argument("null receiver argument");
    sim_of(s).set_receivers(n, i, j);
  });
}

int seiswg_sim_forward(seiswg_sim* s, int32_t isrc, int32_t snap_every, int32_t nfields, const char* const* fields,
                       float* snaps_out, int32_t sync) {
  return guarded([&] {
    seiswg::Sim& sim = sim_of(s);
    if (snap_every > 0 && nfields > 0) {
      if (!fields || !snaps_out) throw std::invalid_argument("null snapshot argument");
      seiswg::Sim::Snapshots snaps;
      snaps.every = snap_every;
      for (int q = 0; q < nfields; ++q) {
        seiswg::StateField f;
        if (!state_field(fields[q], &f)) throw std::invalid_argument(std::string("unknown field ") + fields[q]);
        snaps.fields.push_back(f);
      }
      sim.run_forward(isrc, &snaps);
      const size_t npt = size_t(sim.desc().nx) * sim.desc().nz;
      for (size_t q = 0; q < snaps.frames.size(); ++q)
        std::memcpy(snaps_out + q * npt, snaps.frames[q].data(), npt * sizeof(float));
    } else {
      sim.run_forward(isrc, nullptr);
      if (sync) sim.synchronize();
    }
  });
}

int seiswg_sim_traces(seiswg_sim* s, float* host) {
  return guarded([&] {
    if (!host) throw std::invalid_argument("null buffer");
    sim_of(s).download_traces(host);
  });
}

int seiswg_sim_state(seiswg_sim* s, const char* field, float* host) {
  return guarded([&] {
    seiswg::StateField f;
    if (!host || !state_field(field, &f)) throw std::invalid_argument("unknown field or null buffer");
    sim_of(s).download_state(f, host);
  });
}

int seiswg_sim_kernel_clear(seiswg_sim* s) {
  return guarded([&] { sim_of(s).clear_kmu(); });
}

int seiswg_sim_adjoint_forward(seiswg_sim* s, int32_t isrc, int32_t adj_interval) {
  return guarded([&] { sim_of(s).adjoint_forward(isrc, adj_interval); });
}

int seiswg_sim_adjoint_backward(seiswg_sim* s, const float* adstf, int32_t adj_interval) {
  return guarded([&] {
    if (!adstf && sim_of(s).nrec() > 0) throw std::invalid_argument("null adjoint source");
    sim_of(s).adjoint_backward(adstf, adj_interval);
  });
}

int seiswg_sim_kernel_smooth(seiswg_sim* s, float sigma) {
  return guarded([&] { sim_of(s).smooth_kmu(sigma); });
}

int seiswg_sim_kernel(seiswg_sim* s, float* host) {
  return guarded([&] {
    if (!host) throw std::invalid_argument("null buffer");
    sim_of(s).download_kmu(host);
  });
}

int seiswg_sim_gradient_clear(seiswg_sim* s) {
  return guarded([&] { sim_of(s).gradient_clear(); });
}

int seiswg_sim_forward_op(seiswg_sim* s, int32_t isrc, int32_t ckpt_every) {
  return guarded([&] { sim_of(s).forward_op(isrc, ckpt_every); });
}

int seiswg_sim_backward_op(seiswg_sim* s, const float* adj) {
  return guarded([&] {
    if (!adj && sim_of(s).nrec() > 0) throw std::invalid_argument("null adjoint source");
    sim_of(s).backward_op(adj);
  });
}

int32_t seiswg_sim_checkpoint_interval(const seiswg_sim* s) {
  return s && s->sim ? s->sim->checkpoint_interval() : 0;
}

int seiswg_sim_checkpoint_plan(const seiswg_sim* s, int32_t* slots, int32_t* interval, int64_t* recomputed,
                               size_t* bytes) {
  if (!s || !s->sim) return fail(SEISWG_EINVAL, "null simulation handle");
  if (slots) *slots = s->sim->checkpoint_slots();
  if (interval) *interval = s->sim->checkpoint_interval();
  if (recomputed) *recomputed = s->sim->recompute_steps();
  if (bytes) *bytes = s->sim->checkpoint_bytes();
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_sim_set_observed(seiswg_sim* s, const float* obs) {
  return guarded([&] {
    if (!obs) throw std::invalid_argument("null observed traces");
    sim_of(s).set_observed(obs);
  });
}

int seiswg_sim_misfit_op(seiswg_sim* s, double* J) {
  return guarded([&] {
    if (!J) throw std::invalid_argument("null J");
    *J = sim_of(s).misfit_op();
  });
}

int seiswg_sim_backward_op_device(seiswg_sim* s) {
  return guarded([&] { sim_of(s).backward_op_device(); });
}

int seiswg_sim_gradient(seiswg_sim* s, const char* param, float* host) {
  return guarded([&] {
    if (!param || !host) throw std::invalid_argument("null argument");
    std::string p = param;
    int which = p == "lambda" ? 0 : p == "mu" ? 1 : p == "buoyancy" ? 2 : -1;
    if (which < 0) throw std::invalid_argument("gradient parameter must be lambda, mu or buoyancy");
    sim_of(s).download_gradient(which, host);
  });
}

int seiswg_sim_release_workspace(seiswg_sim* s) {
  return guarded([&] { sim_of(s).release_workspace(); });
}

int seiswg_sim_set_option(seiswg_sim* s, const char* key, int64_t value) {
  return guarded([&] {
    seiswg::Sim& sim = sim_of(s);
    std::string k = key ? key : "";
    if (k == "graphs") sim.set_use_graphs(value != 0);
    else if (k == "chunk_rows") sim.set_chunk_rows(value > 0 ? int(value) : sim.model_chunk_rows());
    else if (k == "loader") sim.set_loader(int(value));
    else if (k == "two_step") sim.set_two_step(value != 0);
    else if (k == "two_step_rows") sim.set_two_step_rows(int(value));
    else if (k == "two_step_producer") sim.set_two_step_producer(value != 0);
    else if (k == "reverse_producer") sim.set_reverse_producer(value != 0);
    else if (k == "cluster") sim.set_use_cluster(value != 0);
    else if (k == "tma") sim.set_use_tma(value != 0);
    else if (k == "autotune") sim.autotune(int(value));
    else if (k == "stability_check") sim.set_stability_check(value != 0);
    else if (k == "pdl") sim.set_pdl(value != 0);
    else if (k == "checkpoint_slots") {
      if (value < 0 || value > (1 << 30)) throw std::invalid_argument("checkpoint_slots out of range");
      sim.set_checkpoint_slots(int(value));
    } else if (k == "checkpoint_budget_mb") {
      if (value < 0) throw std::invalid_argument("checkpoint_budget_mb must be >= 0");
      sim.set_checkpoint_budget(size_t(value) << 20);
    }
    else if (k == "wait_polls") {
      if (value < 0 || value > 0xffffffffLL) throw std::invalid_argument("wait_polls out of range");
      sim.set_wait_polls(unsigned(value));
    } else if (k == "test_arm_extra") {
      if (value < 0 || value > (1 << 20)) throw std::invalid_argument("test_arm_extra out of range");
      sim.set_arm_extra(unsigned(value));
    } else throw std::invalid_argument("unknown option " + k);
  });
}

int seiswg_sim_synchronize(seiswg_sim* s) {
  return guarded([&] { sim_of(s).synchronize(); });
}

uint64_t seiswg_sim_launches(const seiswg_sim* s) { return (s && s->sim) ? s->sim->kernel_launches() : 0; }
void* seiswg_sim_stream(const seiswg_sim* s) { return (s && s->sim) ? static_cast<void*>(s->sim->stream()) : nullptr; }
size_t seiswg_sim_device_bytes(const seiswg_sim* s) { return (s && s->sim) ? s->sim->device_bytes() : 0; }

// ---- batched gradients -----------------------------------------------------------
int seiswg_batch_create(seiswg_sim* const* sims, const float* const* obs, int32_t n, int32_t ckpt_every,
                        void* stream, seiswg_batch** out) {
  if (!sims || !obs || n <= 0 || !out) return fail(SEISWG_EINVAL, "seiswg_batch_create: bad argument");
  *out = nullptr;
  return guarded([&] {
    std::vector<seiswg::BatchProblem> ps;
    for (int p = 0; p < n; ++p) {
      seiswg::Sim& sim = sim_of(sims[p]);
      const auto& d = sim.desc();
      const size_t count = size_t(sim.nsrc()) * (d.psv ? 2 : 1) * sim.nrec() * d.nt;
      if (!obs[p] && count) throw std::invalid_argument("null observed traces");
      ps.push_back(seiswg::BatchProblem{&sim, std::vector<float>(obs[p], obs[p] + count)});
    }
    std::unique_ptr<seiswg_batch> b(new seiswg_batch());
    b->batch.reset(new seiswg::Batch(ps, ckpt_every, static_cast<cudaStream_t>(stream)));
    *out = b.release();
  });
}

int seiswg_batch_run(seiswg_batch* b) {
  if (!b) return fail(SEISWG_EINVAL, "null batch");
  return guarded([&] { b->batch->run(); });
}

int seiswg_batch_set_option(seiswg_batch* b, const char* key, int64_t value) {
  if (!b || !key) return fail(SEISWG_EINVAL, "seiswg_batch_set_option: null argument");
  return guarded([&] {
    const std::string k(key);
    if (k == "chunk_rows") b->batch->set_chunk_rows(int(value));
    else if (k == "autotune") b->batch->autotune(int(value));
    else if (k == "two_step") b->batch->set_two_step(value != 0);
    else if (k == "two_step_recompute") b->batch->set_two_step_recompute(value != 0);
    else if (k == "reverse_producer") b->batch->set_reverse_producer(value != 0);
    else if (k == "concurrent") b->batch->set_concurrent(int(value));
    else if (k == "stream_groups") b->batch->set_stream_groups(int(value));
    else if (k == "tma") b->batch->set_tma(value != 0);
    else if (k == "pdl") b->batch->set_pdl(value != 0);
    else if (k == "queue_wait_us") {
      if (value < 1 || value > (int64_t(1) << 40)) throw std::invalid_argument("queue_wait_us out of range");
      b->batch->set_queue_wait_ns((unsigned long long)value * 1000ull);
    } else if (k == "queue_band") {
      if (value < 0 || value > (1 << 20)) throw std::invalid_argument("queue_band out of range");
      b->batch->set_queue_band(int(value));
    } else if (k == "test_queue_need_extra") {
      if (value < 0 || value > (1 << 30)) throw std::invalid_argument("test_queue_need_extra out of range");
      b->batch->set_queue_need_extra(int(value));
    }
    else if (k == "checkpoint_slots") {
      if (value < 0 || value > (1 << 30)) throw std::invalid_argument("checkpoint_slots out of range");
      b->batch->set_checkpoint_slots(int(value));
    } else throw std::invalid_argument("unknown batch option: " + k);
  });
}

int32_t seiswg_batch_chunk_rows(const seiswg_batch* b) { return b ? b->batch->chunk_rows() : 0; }

int32_t seiswg_batch_two_step(const seiswg_batch* b) { return b && b->batch->two_step() ? 1 : 0; }

int32_t seiswg_batch_concurrent(const seiswg_batch* b) { return b ? b->batch->concurrent() : 0; }

int32_t seiswg_batch_stream_groups(const seiswg_batch* b) { return b ? b->batch->stream_groups() : 0; }

int32_t seiswg_batch_tma_jobs(const seiswg_batch* b) { return b ? b->batch->tma_jobs() : 0; }

int seiswg_batch_queue(const seiswg_batch* b, int64_t* units, int32_t* blocks, int32_t* band) {
  if (!b) return fail(SEISWG_EINVAL, "null batch");
  if (units) *units = b->batch->queue_units();
  if (blocks) *blocks = b->batch->queue_blocks();
  if (band) *band = b->batch->queue_band();
  return SEISWG_OK;
}

int seiswg_batch_checkpoint_plan(const seiswg_batch* b, int32_t* slots, int64_t* recomputed) {
  if (!b) return fail(SEISWG_EINVAL, "null batch");
  return guarded([&] {
    if (slots) *slots = b->batch->checkpoint_slots();
    if (recomputed) *recomputed = b->batch->recompute_steps();
  });
}

int seiswg_batch_gradient(seiswg_batch* b, int32_t problem, const char* param, float* host) {
  if (!b || !param || !host) return fail(SEISWG_EINVAL, "seiswg_batch_gradient: null argument");
  return guarded([&] {
    std::string p = param;
    int which = p == "lambda" ? 0 : p == "mu" ? 1 : p == "buoyancy" ? 2 : -1;
    if (which < 0) throw std::invalid_argument("gradient parameter must be lambda, mu or buoyancy");
    b->batch->download_gradient(problem, which, host);
  });
}

double seiswg_batch_misfit(const seiswg_batch* b, int32_t problem) { return b ? b->batch->misfit(problem) : 0.0; }

int seiswg_batch_info(const seiswg_batch* b, int32_t* jobs, int32_t* slots, uint64_t* launches, size_t* bytes) {
  if (!b) return fail(SEISWG_EINVAL, "null batch");
  if (jobs) *jobs = b->batch->jobs();
  if (slots) *slots = b->batch->slots();
  if (launches) *launches = b->batch->launches_per_run();
  if (bytes) *bytes = b->batch->device_bytes();
  g_last_error.clear();
  return SEISWG_OK;
}

void* seiswg_batch_stream(const seiswg_batch* b) { return b ? static_cast<void*>(b->batch->stream()) : nullptr; }

void seiswg_batch_free(seiswg_batch* b) { delete b; }

// ---- host numerics ------------------------------------------------------------
int seiswg_ricker(int32_t nt, float dt, float f0, float t0, float ang_deg, float amp, float* out) {
  if (nt < 0 || (nt > 0 && !out)) return fail(SEISWG_EINVAL, "seiswg_ricker: bad argument");
  for (int it = 0; it < nt; ++it)
    seiswg::ricker(float(it) * dt, f0, t0, ang_deg, amp, out + it, out + nt + it, out + 2 * nt + it);
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_waveform_misfit(const float* syn, const float* obs, int32_t nrec, int32_t nt, float dt, float* adstf,
                           double* misfit) {
  if (nrec < 0 || nt < 1 || !syn || !obs || !adstf || !misfit)
    return fail(SEISWG_EINVAL, "seiswg_waveform_misfit: bad argument");
  *misfit = seiswg::waveform_misfit(syn, obs, nrec, nt, dt, adstf);
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_npy_encode(const float* data, size_t nrows, size_t ncols, void* out, size_t* len) {
  if (!len || ((nrows * ncols) != 0 && !data)) return fail(SEISWG_EINVAL, "seiswg_npy_encode: bad argument");
  return guarded([&] {
    seiswg::Bytes b = seiswg::make_npy(data, nrows, ncols);
    if (out) {
      if (*len < b.size()) throw std::invalid_argument("output buffer too small");
      std::memcpy(out, b.data(), b.size());
    }
    *len = b.size();
  });
}

int seiswg_l2_misfit(const float* syn, const float* obs, int32_t ntr, int32_t nt, float dt, float* adj, double* J) {
  if (ntr < 0 || nt < 2 || !syn || !obs || !adj || !J) return fail(SEISWG_EINVAL, "seiswg_l2_misfit: bad argument");
  *J = seiswg::l2_misfit(syn, obs, ntr, nt, dt, adj);
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_velocity_gradients(const float* g_lam, const float* g_mu, const float* g_b, const float* vp,
                              const float* vs, const float* rho, size_t n, float* g_vp, float* g_vs, float* g_rho) {
  if (!g_lam || !g_mu || !g_b || !vp || !vs || !rho || !g_vp || !g_vs || !g_rho)
    return fail(SEISWG_EINVAL, "seiswg_velocity_gradients: null argument");
  seiswg::velocity_gradients(g_lam, g_mu, g_b, vp, vs, rho, n, g_vp, g_vs, g_rho);
  g_last_error.clear();
  return SEISWG_OK;
}

int seiswg_infer_grid(const float* x, const float* z, size_t npt, int32_t* nx, int32_t* nz, float* dx, float* dz) {
  if (!x || !z || !nx || !nz || !dx || !dz) return fail(SEISWG_EINVAL, "seiswg_infer_grid: null argument");
  return guarded([&] {
    seiswg::GridInfo g = seiswg::infer_grid(seiswg::ModelData{x, npt}, seiswg::ModelData{z, npt});
    *nx = g.nx;
    *nz = g.nz;
    *dx = g.dx;
    *dz = g.dz;
  });
}

}  // extern "C"
