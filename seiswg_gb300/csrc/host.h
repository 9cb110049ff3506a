// host.h -- the reference-facing host layer: INI configuration, the virtual
// file system, seiswg's file formats and the forward / adjoint workflows.
// This restates, in C++, the behaviour of the reference's Rust host
// (src/config.rs, src/solver.rs, src/main.rs) over the CUDA engine.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"

namespace seiswg {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---- configuration, config.rs:9-57 ---------------------------------------
struct Config {
  std::string workflow;  // "forward" | "adjoint" | "inversion"
  // [solver]
  bool sh = false, psv = true, spin = false;
  uint32_t threads_per_block = 128;
  bool combine_sources = false;
  uint32_t save_snapshot = 0;
  uint32_t adj_interval = 10;
  float smooth = 5.0f;
  uint32_t nt = 0;
  float dt = 0.0f;
  bool abs_left = false, abs_right = false, abs_bottom = false, abs_top = false;
  uint32_t abs_width = 20;
  float abs_alpha = 0.015f;
  // [path]
  std::string output;
  std::string output_traces;  // empty: <output>/traces
  std::string model_true, model_init, sources, stations, traces;
  bool has_output_traces = false, has_model_true = false, has_model_init = false, has_traces = false;
  // [cuda] -- keys the reference ignores
  int chunk_rows = 0;   // 0: engine default
  int graphs = -1;      // -1: engine default, 0 off, 1 on
  int two_step = -1;    // [cuda] two_step: -1 engine default (on for PSV alone), 0 off, 1 on
  // [inversion] -- the workflow the reference lists as planned (README.md:61,
  // main.rs:93-94); keys the reference does not read
  uint32_t inv_iterations = 5;  // descent steps
  float inv_step = 0.02f;       // first relative model change of the line search
  float inv_max_step = 0.1f;    // largest relative model change of a step
  uint32_t inv_trials = 6;      // misfit evaluations per line search
  float inv_smooth = -1.0f;     // gradient smoothing sigma in cells (< 0: [solver] smooth)
  std::string inv_parameters = "vp,vs";  // inverted fields, of vp, vs, rho
};

// config::load (config.rs:118) and config::load_from_str (config.rs:132).
Config config_load(const std::string& path);
Config config_load_str(const std::string& ini_text, const std::string& base_dir);

// ---- VFS, solver.rs:15 -----------------------------------------------------
using Bytes = std::vector<uint8_t>;
using Vfs = std::map<std::string, Bytes>;

// ---- file formats -----------------------------------------------------------
// Model file: int32 npt header + npt f32 (solver.rs:220-233).
std::vector<float> parse_model_bin(const Bytes& b, const std::string& what);
Bytes make_model_bin(const std::vector<float>& data);
// NumPy v1 '<f4' 2-D array (solver.rs:270-301).
Bytes make_npy(const float* data, size_t nrows, size_t ncols);
std::vector<float> parse_npy(const Bytes& b, const std::string& what);
// Whitespace table with '#' comments, bad numbers read as 0 (solver.rs:248-255).
std::vector<std::vector<double>> parse_table(const std::string& text);

// Ricker wavelet (solver.rs:350-356): returns (x, y, z).
void ricker(float t, float f0, float t0, float ang_deg, float amp, float* x, float* y, float* z);
// Waveform misfit and time-reversed adjoint source (solver.rs:432-467).
double waveform_misfit(const float* syn, const float* obs, int nrec, int nt, float dt, float* adstf);
// J = sum (taper * (syn - obs))^2 over ntr traces of nt samples with the
// misfit taper of solver.rs:442-459, and adj = dJ/dsyn (not time-reversed).
double l2_misfit(const float* syn, const float* obs, int ntr, int nt, float dt, float* adj);
// Chain rule from (lambda, mu, buoyancy) gradients to (vp, vs, rho) for
// lambda = rho (vp^2 - 2 vs^2) (0 where vp <= vs), mu = rho vs^2 (fd2d.wgsl:188-201).
void velocity_gradients(const float* g_lam, const float* g_mu, const float* g_b, const float* vp, const float* vs,
                        const float* rho, size_t n, float* g_vp, float* g_vs, float* g_rho);

// Grid inference from coordinate extents (solver.rs:646-656).
struct GridInfo {
  int nx, nz;
  float dx, dz;
};
// Float payload of a model file, read in place (the bytes stay owned by the
// VFS entry or file buffer they come from).
struct ModelData {
  const float* data;
  size_t n;
  size_t size() const { return n; }
  float operator[](size_t k) const { return data[k]; }
};
ModelData view_model_bin(const Bytes& b, const std::string& what);
GridInfo infer_grid(const std::vector<float>& x, const std::vector<float>& z);
GridInfo infer_grid(const ModelData& x, const ModelData& z);
// round(x / dx) as the reference's saturating `as u32` of f32::round.
uint32_t grid_index(float coord, float step);

std::string path_join(const std::string& a, const std::string& b);

// ---- Solver, solver.rs:194-1530 ------------------------------------------
struct SourceDesc {
  int i, j;
  float f0, t0, ang, amp;
};

class Solver {
 public:
  // Solver::new (solver.rs:578).  Inputs are looked up in `vfs` first (key as
  // given, or with a leading "./" removed), then on disk.
  Solver(const Config& cfg, const Vfs& vfs);
  // Solver::run_forward (solver.rs:941).  Outputs are returned and, when
  // write_files is set (the native default), written to disk.
  Vfs run_forward();
  // Solver::run_adjoint (solver.rs:1298).
  Vfs run_adjoint(const Vfs& vfs);
  // `mode = inversion`, which the reference lists as planned (README.md:61)
  // and rejects (main.rs:93-94): steepest descent on the [inversion]
  // parameters from the initial model, each gradient the exact discrete
  // adjoint summed over the shots, smoothed, with a backtracking (Armijo)
  // line search; writes the final model (proc000000_<param>.bin with x, z)
  // to [path] output.  SH or PSV alone.
  Vfs run_inversion(const Vfs& vfs);
  // Misfit J of each accepted or rejected inversion step: (J before, J
  // after, relative step; 0 when rejected).
  struct InversionStep {
    double misfit, new_misfit, step;
    int trials;
    bool accepted;
  };
  const std::vector<InversionStep>& inversion_history() const { return inv_history_; }

  void set_write_files(bool on) { write_files_ = on; }
  Sim& sim() { return *sim_; }
  const Config& config() const { return cfg_; }
  int nx() const { return grid_.nx; }
  int nz() const { return grid_.nz; }
  float dx() const { return grid_.dx; }
  float dz() const { return grid_.dz; }
  int nrec() const { return int(rec_i_.size()); }
  int nsrc() const { return int(srcs_.size()); }
  const std::vector<double>& misfits() const { return misfits_; }
  double total_misfit() const { return total_misfit_; }

 private:
  Bytes lookup(const Vfs& vfs, const std::string& path) const;
  // The VFS entry itself, or the file read into `hold` when the VFS lacks it.
  const Bytes& lookup_ref(const Vfs& vfs, const std::string& path, Bytes& hold) const;
  void write_file(const std::string& path, const Bytes& b) const;

  Config cfg_;
  GridInfo grid_{};
  std::vector<SourceDesc> srcs_;
  std::vector<int> rec_i_, rec_j_;
  std::unique_ptr<Sim> sim_;
  bool write_files_ = true;
  std::vector<double> misfits_;
  double total_misfit_ = 0.0;
  std::vector<InversionStep> inv_history_;
};

// Logging (env RUST_LOG-like level via SEISWG_LOG: error|warn|info; default info).
void log_info(const std::string& msg);

}  // namespace seiswg
