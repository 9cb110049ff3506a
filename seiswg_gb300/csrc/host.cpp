// host.cpp -- configuration, file formats, VFS and the forward / adjoint
// workflows of seiswg (src/config.rs, src/solver.rs), over the CUDA engine.
#include "host.h"

#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <list>
#include <sstream>
#include <system_error>
#include <limits>
#include <thread>

namespace seiswg {

namespace {

constexpr float kPi = 3.14159265358979323846f;

std::string lower(std::string s) {
  for (char& c : s) c = char(std::tolower(static_cast<unsigned char>(c)));
  return s;
}

std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
  while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
  return s.substr(a, b - a);
}

std::string fmt6(uint32_t v) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%06u", v);
  return buf;
}

bool file_exists(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0;
}

void mkdirs(const std::string& path) {
  if (path.empty()) return;
  std::string cur;
  size_t pos = 0;
  while (pos <= path.size()) {
    size_t nxt = path.find('/', pos);
    if (nxt == std::string::npos) nxt = path.size();
    cur = path.substr(0, nxt);
    if (!cur.empty() && !file_exists(cur)) {
      if (::mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST)
        throw Error("Cannot create directory " + cur + ": " + std::strerror(errno));
    }
    pos = nxt + 1;
  }
}

Bytes read_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error("Cannot read " + path);
  return Bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// ---- INI (configparser 3.x semantics as used by config.rs) ----------------
// Sections and keys are case-insensitive; ';' and '#' start a comment; '=' or
// ':' separate key and value; a key without a delimiter has no value.
using Ini = std::map<std::string, std::map<std::string, std::pair<bool, std::string>>>;

Ini parse_ini(const std::string& text) {
  Ini ini;
  std::string section = "default";
  std::istringstream in(text);
  std::string raw;
  int num = 0;
  while (std::getline(in, raw)) {
    ++num;
    size_t c = raw.find_first_of(";#");
    std::string line = trim(c == std::string::npos ? raw : raw.substr(0, c));
    if (line.empty()) continue;
    if (line[0] == '[') {
      size_t e = line.rfind(']');
      if (e == std::string::npos)
        throw Error("line " + std::to_string(num) + ": Found opening bracket for section name but no closing bracket");
      section = lower(trim(line.substr(1, e - 1)));
      continue;
    }
    if (line[0] == '=' || line[0] == ':')
      throw Error("line " + std::to_string(num) + ": Started with a delimiter but no key");
    size_t d = line.find_first_of("=:");
    auto& sec = ini[section];
    if (d == std::string::npos) {
      sec[lower(line)] = {false, ""};
    } else {
      std::string key = lower(trim(line.substr(0, d)));
      if (key.empty()) throw Error("line " + std::to_string(num) + ": Key cannot be empty");
      sec[key] = {true, trim(line.substr(d + 1))};
    }
  }
  return ini;
}

bool ini_get(const Ini& ini, const std::string& sec, const std::string& key, std::string* out) {
  auto s = ini.find(lower(sec));
  if (s == ini.end()) return false;
  auto k = s->second.find(lower(key));
  if (k == s->second.end() || !k->second.first) return false;
  *out = k->second.second;
  return true;
}

std::string get_required(const Ini& ini, const std::string& sec, const std::string& key) {
  std::string v;
  if (!ini_get(ini, sec, key, &v)) throw Error("[" + sec + "] " + key + " is required");
  return v;
}

bool get_bool(const Ini& ini, const std::string& sec, const std::string& key, bool def) {
  std::string v;
  if (!ini_get(ini, sec, key, &v)) return def;
  return lower(trim(v)) == "yes";  // config.rs:72-76: only "yes" is true
}

bool parse_u32(const std::string& s, uint32_t* out) {
  std::string t = trim(s);
  if (t.empty()) return false;
  size_t i = (t[0] == '+') ? 1 : 0;
  if (i == t.size()) return false;
  uint64_t v = 0;
  for (; i < t.size(); ++i) {
    if (t[i] < '0' || t[i] > '9') return false;
    v = v * 10 + uint64_t(t[i] - '0');
    if (v > 0xffffffffull) return false;
  }
  *out = uint32_t(v);
  return true;
}

bool parse_f32(const std::string& s, float* out) {
  std::string t = trim(s);
  if (t.empty()) return false;
  char* end = nullptr;
  errno = 0;
  float v = std::strtof(t.c_str(), &end);
  if (end != t.c_str() + t.size()) return false;
  *out = v;
  return true;
}

uint32_t get_u32(const Ini& ini, const std::string& sec, const std::string& key) {
  uint32_t v;
  if (!parse_u32(get_required(ini, sec, key), &v)) throw Error("[" + sec + "] " + key + " must be an integer");
  return v;
}

uint32_t get_u32_or(const Ini& ini, const std::string& sec, const std::string& key, uint32_t def) {
  std::string s;
  uint32_t v;
  return (ini_get(ini, sec, key, &s) && parse_u32(s, &v)) ? v : def;
}

float get_f32(const Ini& ini, const std::string& sec, const std::string& key) {
  float v;
  if (!parse_f32(get_required(ini, sec, key), &v)) throw Error("[" + sec + "] " + key + " must be a float");
  return v;
}

float get_f32_or(const Ini& ini, const std::string& sec, const std::string& key, float def) {
  std::string s;
  float v;
  return (ini_get(ini, sec, key, &s) && parse_f32(s, &v)) ? v : def;
}

// config.rs:105-112: paths are relative to the directory of the config file.
std::string resolve(const std::string& base, const std::string& raw) {
  std::string p = trim(raw);
  if (!p.empty() && p[0] == '/') return p;
  return path_join(base, p);
}

Config parse_config(const Ini& ini, const std::string& base) {
  Config c;
  c.workflow = lower(trim(get_required(ini, "workflow", "mode")));
  c.nt = get_u32(ini, "solver", "nt");
  c.dt = get_f32(ini, "solver", "dt");
  c.abs_left = get_bool(ini, "solver", "abs_left", false);
  c.abs_right = get_bool(ini, "solver", "abs_right", false);
  c.abs_bottom = get_bool(ini, "solver", "abs_bottom", false);
  c.abs_top = get_bool(ini, "solver", "abs_top", false);
  c.abs_width = get_u32_or(ini, "solver", "abs_width", 20);
  c.abs_alpha = get_f32_or(ini, "solver", "abs_alpha", 0.015f);
  c.sh = get_bool(ini, "solver", "sh", false);
  c.psv = get_bool(ini, "solver", "psv", true);
  c.spin = get_bool(ini, "solver", "spin", false);
  c.threads_per_block = get_u32_or(ini, "solver", "threads_per_block", 128);
  c.combine_sources = get_bool(ini, "solver", "combine_sources", false);
  c.save_snapshot = get_u32_or(ini, "solver", "save_snapshot", 0);
  c.adj_interval = get_u32_or(ini, "solver", "adj_interval", 10);
  c.smooth = get_f32_or(ini, "solver", "smooth", 5.0f);
  std::string v;
  c.output = resolve(base, get_required(ini, "path", "output"));
  if ((c.has_output_traces = ini_get(ini, "path", "output_traces", &v))) c.output_traces = resolve(base, v);
  if ((c.has_model_true = ini_get(ini, "path", "model_true", &v))) c.model_true = resolve(base, v);
  if ((c.has_model_init = ini_get(ini, "path", "model_init", &v))) c.model_init = resolve(base, v);
  c.sources = resolve(base, get_required(ini, "path", "sources"));
  c.stations = resolve(base, get_required(ini, "path", "stations"));
  if ((c.has_traces = ini_get(ini, "path", "traces", &v))) c.traces = resolve(base, v);
  uint32_t u;
  if (ini_get(ini, "cuda", "chunk_rows", &v) && parse_u32(v, &u)) c.chunk_rows = int(u);
  if (ini_get(ini, "cuda", "graphs", &v)) c.graphs = lower(trim(v)) == "yes" ? 1 : 0;
  if (ini_get(ini, "cuda", "two_step", &v)) c.two_step = lower(trim(v)) == "yes" ? 1 : 0;
  c.inv_iterations = get_u32_or(ini, "inversion", "iterations", c.inv_iterations);
  c.inv_step = get_f32_or(ini, "inversion", "step", c.inv_step);
  c.inv_max_step = get_f32_or(ini, "inversion", "max_step", c.inv_max_step);
  c.inv_trials = get_u32_or(ini, "inversion", "line_search_trials", c.inv_trials);
  c.inv_smooth = get_f32_or(ini, "inversion", "smooth", c.inv_smooth);
  if (ini_get(ini, "inversion", "parameters", &v)) c.inv_parameters = lower(trim(v));
  return c;
}

}  // namespace

std::string path_join(const std::string& a, const std::string& b) {
  if (b.empty()) return a;
  if (!b.empty() && b[0] == '/') return b;
  if (a.empty()) return b;
  if (a.back() == '/') return a + b;
  return a + "/" + b;
}

Config config_load(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error("Cannot open " + path + ": No such file or directory");
  std::string text((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  size_t slash = path.rfind('/');
  std::string base = slash == std::string::npos ? std::string() : path.substr(0, slash == 0 ? 1 : slash);
  return parse_config(parse_ini(text), base);
}

Config config_load_str(const std::string& text, const std::string& base_dir) {
  return parse_config(parse_ini(text), base_dir);
}

// ---- file formats -----------------------------------------------------------
std::vector<float> parse_model_bin(const Bytes& b, const std::string& what) {
  if (b.size() < 4) throw Error("Model file too small: " + what);
  int32_t n;
  std::memcpy(&n, b.data(), 4);
  if (n < 0) throw Error("Model file " + what + " has a negative point count");
  size_t expected = 4 + size_t(n) * 4;
  if (b.size() < expected)
    throw Error("Model file " + what + " too short (expected " + std::to_string(expected) + " bytes, got " +
                std::to_string(b.size()) + ")");
  std::vector<float> out(static_cast<size_t>(n));
  std::memcpy(out.data(), b.data() + 4, size_t(n) * 4);
  return out;
}

ModelData view_model_bin(const Bytes& b, const std::string& what) {
  if (b.size() < 4) throw Error("Model file too small: " + what);
  int32_t n;
  std::memcpy(&n, b.data(), 4);
  if (n < 0) throw Error("Model file " + what + " has a negative point count");
  const size_t expected = 4 + size_t(n) * 4;
  if (b.size() < expected)
    throw Error("Model file " + what + " too short (expected " + std::to_string(expected) + " bytes, got " +
                std::to_string(b.size()) + ")");
  // The payload follows the 4-byte header: 4-byte aligned floats, read in place.
  return ModelData{reinterpret_cast<const float*>(b.data() + 4), size_t(n)};
}

Bytes make_model_bin(const std::vector<float>& d) {
  Bytes out(4 + d.size() * 4);
  int32_t n = int32_t(d.size());
  std::memcpy(out.data(), &n, 4);
  std::memcpy(out.data() + 4, d.data(), d.size() * 4);
  return out;
}

// solver.rs:270-285: header dict padded with spaces so that dict + '\n' is a
// multiple of 64 bytes.
Bytes make_npy(const float* data, size_t nrows, size_t ncols) {
  std::string dict = "{'descr': '<f4', 'fortran_order': False, 'shape': (" + std::to_string(nrows) + ", " +
                     std::to_string(ncols) + "), }";
  size_t header_len = (dict.size() + 1 + 63) / 64 * 64;
  std::string header = dict;
  while (header.size() < header_len - 1) header.push_back(' ');
  header.push_back('\n');
  Bytes out;
  out.reserve(10 + header_len + nrows * ncols * 4);
  const char magic[] = "\x93NUMPY\x01\x00";
  out.insert(out.end(), magic, magic + 8);
  uint16_t hl = uint16_t(header_len);
  out.push_back(uint8_t(hl & 0xff));
  out.push_back(uint8_t(hl >> 8));
  out.insert(out.end(), header.begin(), header.end());
  const uint8_t* p = reinterpret_cast<const uint8_t*>(data);
  out.insert(out.end(), p, p + nrows * ncols * 4);
  return out;
}

std::vector<float> parse_npy(const Bytes& b, const std::string& what) {
  if (b.size() < 10 || std::memcmp(b.data(), "\x93NUMPY", 6) != 0) throw Error("Not a NumPy file: " + what);
  size_t hl = size_t(b[8]) | (size_t(b[9]) << 8);
  size_t start = 10 + hl;
  if (b.size() < start) throw Error("Truncated .npy header in " + what);
  if ((b.size() - start) % 4 != 0) throw Error("Payload length not a multiple of 4 in " + what);
  std::vector<float> out(static_cast<size_t>((b.size() - start) / 4));
  std::memcpy(out.data(), b.data() + start, out.size() * 4);
  return out;
}

std::vector<std::vector<double>> parse_table(const std::string& text) {
  std::vector<std::vector<double>> rows;
  std::istringstream in(text);
  std::string line;
  while (std::getline(in, line)) {
    std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    std::istringstream ls(t);
    std::string tok;
    std::vector<double> row;
    while (ls >> tok) {
      char* end = nullptr;
      double v = std::strtod(tok.c_str(), &end);
      row.push_back(end == tok.c_str() + tok.size() ? v : 0.0);  // unwrap_or(0.0)
    }
    rows.push_back(row);
  }
  return rows;
}

void ricker(float t, float f0, float t0, float ang_deg, float amp, float* x, float* y, float* z) {
  const float a = (kPi * f0) * (kPi * f0);
  const float d = t - t0;
  const float stf = -amp * (1.0f - 2.0f * a * d * d) * std::exp(-a * d * d);
  const float ang = ang_deg * (kPi / 180.0f);  // f32::to_radians
  *x = stf * std::sin(ang);
  *y = stf;
  *z = -stf * std::cos(ang);
}

double waveform_misfit(const float* syn, const float* obs, int nrec, int nt, float dt, float* adstf) {
  double misfit = 0.0;
  const float t_end = float(nt - 1) * dt;
  const float tw = t_end / 10.0f;
  const float t_min = tw, t_max = t_end - tw;
  for (int ir = 0; ir < nrec; ++ir) {
    for (int it = 0; it < nt; ++it) {
      const size_t kt = size_t(ir) * nt + it;
      const size_t akt = size_t(ir) * nt + (nt - 1 - it);
      const float t = float(it) * dt;
      float taper = 1.0f;
      if (t <= t_min) taper = 0.5f + 0.5f * std::cos(kPi * (t_min - t) / tw);
      else if (t >= t_max) taper = 0.5f + 0.5f * std::cos(kPi * (t_max - t) / tw);
      const float diff = (syn[kt] - obs[kt]) * taper;
      misfit += double(diff) * double(diff);
      adstf[akt] = diff * taper * 2.0f;
    }
  }
  return std::sqrt(misfit);
}

double l2_misfit(const float* syn, const float* obs, int ntr, int nt, float dt, float* adj) {
  // Taper of solver.rs:442-459, in double here.
  const double t_end = double(nt - 1) * double(dt), tw = t_end / 10.0, pi = 3.14159265358979323846;
  double sum = 0.0;
  for (int it = 0; it < nt; ++it) {
    const double t = double(it) * double(dt);
    double tau = 1.0;
    if (t <= tw) tau = 0.5 + 0.5 * std::cos(pi * (tw - t) / tw);
    else if (t >= t_end - tw) tau = 0.5 + 0.5 * std::cos(pi * ((t_end - tw) - t) / tw);
    for (int r = 0; r < ntr; ++r) {
      const size_t k = size_t(r) * nt + it;
      const double d = (double(syn[k]) - double(obs[k])) * tau;
      sum += d * d;
      if (adj) adj[k] = float(2.0 * d * tau);
    }
  }
  return sum;
}

void velocity_gradients(const float* g_lam, const float* g_mu, const float* g_b, const float* vp, const float* vs,
                        const float* rho, size_t n, float* g_vp, float* g_vs, float* g_rho) {
  for (size_t k = 0; k < n; ++k) {
    const double a = vp[k], b = vs[k], r = rho[k], gl = g_lam[k], gm = g_mu[k], gb = g_b[k];
    const bool live = a > b;  // vps2lm sets lambda to 0 otherwise (fd2d.wgsl:196-200)
    g_vp[k] = float(live ? gl * 2.0 * r * a : 0.0);
    g_vs[k] = float((live ? gl * (-4.0 * r * b) : 0.0) + gm * 2.0 * r * b);
    g_rho[k] = float((live ? gl * (a * a - 2.0 * b * b) : 0.0) + gm * b * b - gb / (r * r));
  }
}

namespace {

// The grid read from the layout itself (k = i*nz + j, z fastest): nz is the
// length of the first run of equal x, nx = npt / nz, and every run must
// repeat the first run's z values at one x.  Returns false when the
// coordinates do not form such a grid.
bool grid_from_layout(const ModelData& x, const ModelData& z, GridInfo& g) {
  const size_t npt = x.size();
  size_t nz = 1;
  while (nz < npt && x[nz] == x[0]) ++nz;
  if (nz < 2 || npt % nz != 0 || npt / nz < 2) return false;
  const size_t nx = npt / nz;
  for (size_t i = 0; i < nx; ++i) {
    const float xi = x[i * nz];
    if (i > 0 && !(xi > x[(i - 1) * nz])) return false;
    for (size_t j = 0; j < nz; ++j)
      if (x[i * nz + j] != xi || z[i * nz + j] != z[j]) return false;
  }
  for (size_t j = 1; j < nz; ++j)
    if (!(z[j] > z[j - 1])) return false;
  g.nx = int(nx);
  g.nz = int(nz);
  g.dx = (x[(nx - 1) * nz] - x[0]) / float(nx - 1);
  g.dz = (z[nz - 1] - z[0]) / float(nz - 1);
  return true;
}

}  // namespace

// max - min of n > 0 floats, as the reference folds them (solver.rs:647-650:
// f32::max from -infinity, f32::min from +infinity): NaN elements are passed
// over wherever they are, the first included.  Every partial minimum and
// maximum starts from +/-infinity and takes an element only when it compares
// below / above, which a NaN never does.  Coordinate files of large grids
// (4096 x 4096: 64 MB each) are scanned by up to 16 threads over contiguous
// parts, each in 16 independent lanes that the compiler vectorises.
namespace {
float extent_of(const float* v, size_t n) {
  struct MinMax {
    float lo, hi;
  };
  auto scan = [](const float* p, size_t m) {
    constexpr int W = 16;
    float lo[W], hi[W];
    for (int q = 0; q < W; ++q) {
      lo[q] = std::numeric_limits<float>::infinity();
      hi[q] = -std::numeric_limits<float>::infinity();
    }
    const size_t mw = m / W * W;
    for (size_t k = 0; k < mw; k += W)
      for (int q = 0; q < W; ++q) {
        const float a = p[k + q];
        lo[q] = a < lo[q] ? a : lo[q];
        hi[q] = hi[q] < a ? a : hi[q];
      }
    for (size_t k = mw; k < m; ++k) {
      lo[0] = p[k] < lo[0] ? p[k] : lo[0];
      hi[0] = hi[0] < p[k] ? p[k] : hi[0];
    }
    MinMax r{lo[0], hi[0]};
    for (int q = 1; q < W; ++q) {
      r.lo = lo[q] < r.lo ? lo[q] : r.lo;
      r.hi = r.hi < hi[q] ? hi[q] : r.hi;
    }
    return r;
  };
  const size_t kPart = size_t(1) << 20;  // elements per thread at least
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned nth = unsigned(std::min<size_t>({size_t(16), size_t(hw), (n + kPart - 1) / kPart}));
  std::vector<MinMax> part(nth);
  const size_t per = (n + nth - 1) / nth;
  auto bounds = [&](unsigned t) {
    const size_t b = std::min(n, size_t(t) * per);
    return std::make_pair(b, std::min(n, b + per));
  };
  // Parts 1.. go to threads as long as threads can be started; this thread
  // scans part 0 and every part no thread took.
  std::vector<std::thread> pool;
  unsigned handed = 1;
  for (; handed < nth; ++handed) {
    const auto [b, e] = bounds(handed);
    const unsigned t = handed;
    try {
      pool.emplace_back([&part, &scan, v, t, b = b, e = e] { part[t] = scan(v + b, e - b); });
    } catch (const std::system_error&) {
      break;
    }
  }
  for (unsigned t = 0; t < nth; ++t)
    if (t == 0 || t >= handed) {
      const auto [b, e] = bounds(t);
      part[t] = scan(v + b, e - b);
    }
  for (std::thread& th : pool) th.join();
  MinMax r = part[0];
  for (unsigned t = 1; t < nth; ++t) {
    r.lo = part[t].lo < r.lo ? part[t].lo : r.lo;
    r.hi = r.hi < part[t].hi ? part[t].hi : r.hi;
  }
  return r.hi - r.lo;
}
}  // namespace

GridInfo infer_grid(const std::vector<float>& x, const std::vector<float>& z) {
  if (x.size() != z.size()) throw Error("coordinate files are empty or differ in size");
  return infer_grid(ModelData{x.data(), x.size()}, ModelData{z.data(), z.size()});
}

GridInfo infer_grid(const ModelData& x, const ModelData& z) {
  if (x.size() == 0 || z.size() == 0 || x.size() != z.size()) throw Error("coordinate files are empty or differ in size");
  const float lx = extent_of(x.data, x.size()), lz = extent_of(z.data, z.size());
  if (!(lx > 0.0f) || !(lz > 0.0f)) throw Error("coordinate extents must be positive");
  // The reference's rule (solver.rs:646-656): nx, nz from npt and the extents'
  // aspect ratio, which holds for square cells (dx == dz).
  const double npt = double(x.size());
  GridInfo g;
  g.nx = int(std::round(std::sqrt(npt * double(lx) / double(lz))));
  g.nz = int(std::round(std::sqrt(npt * double(lz) / double(lx))));
  // Accepted when it tiles npt and agrees with the layout's first run of
  // equal x (nz values, then a new x): O(1), without scanning the layout.
  if (g.nx >= 2 && g.nz >= 2 && size_t(g.nx) * size_t(g.nz) == x.size() && x[size_t(g.nz) - 1] == x[0] &&
      x[size_t(g.nz)] != x[0]) {
    g.dx = lx / float(g.nx - 1);
    g.dz = lz / float(g.nz - 1);
    return g;
  }
  GridInfo lay{};
  const bool have_layout = grid_from_layout(x, z, lay);
  // Rectangular cells (dx != dz), where the aspect-ratio rule cannot work:
  // the grid read from the coordinate layout.
  if (have_layout) return lay;
  // Otherwise the reference's result wherever it tiles npt, as the reference
  // itself takes it without looking at the layout (coordinates stored z
  // first, or x values that differ by rounding within a column).
  if (g.nx >= 2 && g.nz >= 2 && size_t(g.nx) * size_t(g.nz) == x.size()) {
    log_info("grid inferred from the coordinate extents (" + std::to_string(g.nx) + " x " + std::to_string(g.nz) +
             "); the coordinates do not follow the layout k = i*nz + j exactly");
    g.dx = lx / float(g.nx - 1);
    g.dz = lz / float(g.nz - 1);
    return g;
  }
  throw Error("cannot infer a rectangular grid from the coordinates (nx=" + std::to_string(g.nx) +
              ", nz=" + std::to_string(g.nz) + ", npt=" + std::to_string(x.size()) + ")");
}

uint32_t grid_index(float coord, float step) {
  float r = std::round(coord / step);
  if (!(r > 0.0f)) return 0;                 // saturating cast: negative and NaN -> 0
  if (r >= 4294967295.0f) return 0xffffffffu;
  return uint32_t(r);
}

void log_info(const std::string& msg) {
  const char* lvl = std::getenv("SEISWG_LOG");
  if (lvl && (std::strcmp(lvl, "error") == 0 || std::strcmp(lvl, "warn") == 0 || std::strcmp(lvl, "off") == 0)) return;
  std::fprintf(stderr, "[seiswg] %s\n", msg.c_str());
}

// ---- Solver ----------------------------------------------------------------
Bytes Solver::lookup(const Vfs& vfs, const std::string& path) const {
  Bytes hold;
  const Bytes& b = lookup_ref(vfs, path, hold);
  return &b == &hold ? std::move(hold) : b;
}

const Bytes& Solver::lookup_ref(const Vfs& vfs, const std::string& path, Bytes& hold) const {
  auto it = vfs.find(path);
  if (it == vfs.end() && path.rfind("./", 0) == 0) it = vfs.find(path.substr(2));
  if (it != vfs.end()) return it->second;
  hold = read_file(path);
  return hold;
}

void Solver::write_file(const std::string& path, const Bytes& b) const {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw Error("Cannot create " + path);
  f.write(reinterpret_cast<const char*>(b.data()), std::streamsize(b.size()));
  if (!f) throw Error("Cannot write " + path);
}

Solver::Solver(const Config& cfg, const Vfs& vfs) : cfg_(cfg) {
  const std::string model_dir = cfg.has_model_init ? cfg.model_init : cfg.has_model_true ? cfg.model_true : "";
  if (!cfg.has_model_init && !cfg.has_model_true) throw Error("No model path in config");
  const bool spin = cfg.spin;
  // Model files are read in place from the VFS (files not in the VFS are
  // read from disk into `held`): no copies of the fields on the host.
  std::list<Bytes> held;
  auto load = [&](const std::string& name) {
    std::string p = path_join(model_dir, "proc000000_" + name + ".bin");
    Bytes hold;
    const Bytes& b = lookup_ref(vfs, p, hold);
    if (&b == &hold) {
      held.push_back(std::move(hold));
      return view_model_bin(held.back(), p);
    }
    return view_model_bin(b, p);
  };
  ModelData rho = load("rho");
  const size_t npt = rho.size();
  ModelData x = load("x"), z = load("z");
  if (x.size() != npt || z.size() != npt) throw Error("coordinate files do not match the model size");
  grid_ = infer_grid(x, z);
  {
    char buf[160];
    std::snprintf(buf, sizeof buf, "Grid: nx=%d nz=%d npt=%zu dx=%.1f dz=%.1f", grid_.nx, grid_.nz, npt, grid_.dx,
                  grid_.dz);
    log_info(buf);
  }

  // Sources (solver.rs:703-733).
  const int nt = int(cfg.nt);
  const Bytes src_bytes = lookup(vfs, cfg.sources);
  auto src_rows = parse_table(std::string(reinterpret_cast<const char*>(src_bytes.data()), src_bytes.size()));
  std::vector<int> si, sj;
  for (size_t s = 0; s < src_rows.size(); ++s) {
    const auto& r = src_rows[s];
    auto g = [&](size_t q, double def) { return q < r.size() ? r[q] : def; };
    SourceDesc sd;
    const float sx = float(g(0, 0.0)), sz = float(g(1, 0.0));
    sd.f0 = float(g(3, 10.0));
    sd.t0 = float(g(4, 0.1));
    sd.ang = float(g(5, 0.0));
    sd.amp = float(g(6, 1.0e10));
    uint32_t ix = grid_index(sx, grid_.dx), iz = grid_index(sz, grid_.dz);
    if (ix >= uint32_t(grid_.nx) || iz >= uint32_t(grid_.nz))
      throw Error("source " + std::to_string(s) + " at (" + std::to_string(sx) + ", " + std::to_string(sz) +
                  ") lies outside the grid");
    sd.i = int(ix);
    sd.j = int(iz);
    srcs_.push_back(sd);
    si.push_back(sd.i);
    sj.push_back(sd.j);
  }
  const size_t nsrc = srcs_.size();
  std::vector<float> stf(3 * nsrc * size_t(nt));
  for (size_t s = 0; s < nsrc; ++s) {
    for (int it = 0; it < nt; ++it) {
      float a, b, c;
      ricker(float(it) * cfg.dt, srcs_[s].f0, srcs_[s].t0, srcs_[s].ang, srcs_[s].amp, &a, &b, &c);
      stf[(0 * nsrc + s) * nt + it] = a;
      stf[(1 * nsrc + s) * nt + it] = b;
      stf[(2 * nsrc + s) * nt + it] = c;
    }
  }

  // Stations (solver.rs:742-751).
  Bytes st = lookup(vfs, cfg.stations);
  auto rec_rows = parse_table(std::string(reinterpret_cast<const char*>(st.data()), st.size()));
  for (size_t r = 0; r < rec_rows.size(); ++r) {
    const auto& row = rec_rows[r];
    const float rx = float(row.size() > 0 ? row[0] : 0.0), rz = float(row.size() > 1 ? row[1] : 0.0);
    uint32_t ix = grid_index(rx, grid_.dx), iz = grid_index(rz, grid_.dz);
    if (ix >= uint32_t(grid_.nx) || iz >= uint32_t(grid_.nz))
      throw Error("station " + std::to_string(r) + " at (" + std::to_string(rx) + ", " + std::to_string(rz) +
                  ") lies outside the grid");
    rec_i_.push_back(int(ix));
    rec_j_.push_back(int(iz));
  }
  // Remaining model fields (solver.rs:626-638, 661-675): spin models carry
  // lambda/mu directly, the others vp/vs.
  std::vector<std::pair<ModelField, ModelData>> fields;
  fields.emplace_back(ModelField::RHO, rho);
  if (spin) {
    fields.emplace_back(ModelField::LAMBDA, load("lambda"));
    fields.emplace_back(ModelField::MU, load("mu"));
    fields.emplace_back(ModelField::NU, load("nu"));
    fields.emplace_back(ModelField::J, load("j"));
    fields.emplace_back(ModelField::LAMBDA_C, load("lambda_c"));  // read as the reference does; unused
    fields.emplace_back(ModelField::MU_C, load("mu_c"));
    fields.emplace_back(ModelField::NU_C, load("nu_c"));
  } else {
    fields.emplace_back(ModelField::VP, load("vp"));
    fields.emplace_back(ModelField::VS, load("vs"));
  }
  for (const auto& f : fields)
    if (f.second.size() != npt) throw Error("a model file does not match the density size");

  // All inputs are read and checked; only now is the GPU touched.
  SimDesc d;
  d.nx = grid_.nx;
  d.nz = grid_.nz;
  d.nt = int(cfg.nt);
  d.dx = grid_.dx;
  d.dz = grid_.dz;
  d.dt = cfg.dt;
  d.sh = cfg.sh;
  d.psv = cfg.psv;
  d.spin = cfg.spin;
  d.abs_left = cfg.abs_left;
  d.abs_right = cfg.abs_right;
  d.abs_bottom = cfg.abs_bottom;
  d.abs_top = cfg.abs_top;
  d.abs_width = int(cfg.abs_width);
  d.abs_alpha = cfg.abs_alpha;
  sim_.reset(new Sim(d));
  if (cfg.chunk_rows > 0) sim_->set_chunk_rows(cfg.chunk_rows);
  if (cfg.graphs >= 0) sim_->set_use_graphs(cfg.graphs == 1);
  if (cfg.two_step >= 0) sim_->set_two_step(cfg.two_step == 1);
  for (const auto& f : fields) {
    const bool spin_only = f.first == ModelField::NU || f.first == ModelField::J || f.first == ModelField::MU_C ||
                           f.first == ModelField::NU_C;
    if (spin_only && !cfg.psv) continue;  // the SH system has no micropolar fields
    sim_->upload_model(f.first, f.second.data);
  }
  sim_->prepare_model();

  sim_->set_sources(int(nsrc), si.data(), sj.data(), stf.data());
  sim_->set_receivers(int(rec_i_.size()), rec_i_.data(), rec_j_.data());
}

Vfs Solver::run_forward() {
  Vfs out;
  const bool sh = cfg_.sh, psv = cfg_.psv, spin = cfg_.spin && cfg_.psv;
  const int nt = int(cfg_.nt), nrec = this->nrec();
  const uint32_t snap = cfg_.save_snapshot;
  const std::string trace_dir = cfg_.has_output_traces ? cfg_.output_traces : path_join(cfg_.output, "traces");
  if (write_files_) {
    mkdirs(trace_dir);
    if (snap > 0) mkdirs(cfg_.output);
  }
  std::vector<std::pair<int, int>> runs;
  if (cfg_.combine_sources) runs.push_back({-1, 0});
  else for (int s = 0; s < nsrc(); ++s) runs.push_back({s, s});

  std::map<std::string, std::vector<float>> snap_bufs;
  uint32_t snap_count = 0;
  // The trace components written out: uy (1) for SH; ux, uz (0, 2) for PSV;
  // with spin also ry, yi (1, 3).  Only those are copied back, into a buffer
  // whose other components are never read (left uninitialised).
  const unsigned comps = (sh ? 1u << 1 : 0u) | (psv ? (1u << 0) | (1u << 2) : 0u) | (spin ? (1u << 1) | (1u << 3) : 0u);
  std::unique_ptr<float[]> obs(new float[size_t(5) * nrec * nt]);
  for (auto [isrc, idx] : runs) {
    log_info("Forward run  isrc=" + (isrc < 0 ? std::string("all") : std::to_string(isrc)) + "  (" +
             std::to_string(nt) + " time steps)");
    Sim::Snapshots snaps;
    snaps.every = int(snap);
    std::vector<std::string> names;
    if (snap > 0) {
      if (sh) { snaps.fields.push_back(StateField::VY); names.push_back("vy"); }
      if (psv) {
        snaps.fields.push_back(StateField::VX); names.push_back("vx");
        snaps.fields.push_back(StateField::VZ); names.push_back("vz");
        if (spin) { snaps.fields.push_back(StateField::VYC); names.push_back("ry"); }
      }
    }
    sim_->run_forward(isrc, snap > 0 ? &snaps : nullptr);
    // Snapshots (solver.rs:1035-1038, 1144-1176).
    const size_t nf = snaps.fields.size();
    for (size_t q = 0; q < snaps.steps.size(); ++q) {
      for (size_t f = 0; f < nf; ++f) {
        const std::vector<float>& fr = snaps.frames[q * nf + f];
        auto& acc = snap_bufs[names[f]];
        acc.insert(acc.end(), fr.begin(), fr.end());
        if (write_files_) {
          const uint8_t* p = reinterpret_cast<const uint8_t*>(fr.data());
          write_file(path_join(cfg_.output, "proc" + fmt6(uint32_t(snaps.steps[q])) + "_" + names[f] + ".bin"),
                     Bytes(p, p + fr.size() * 4));
        }
      }
      ++snap_count;
    }
    // Traces (solver.rs:1047-1101).
    sim_->download_traces(obs.get(), comps);
    const size_t nobs = size_t(nrec) * nt;
    auto emit = [&](const std::string& name, int comp, bool npy) {
      const float* c = obs.get() + size_t(comp) * nobs;
      std::string p = path_join(trace_dir, name + "_" + fmt6(uint32_t(idx)) + ".npy");
      Bytes b = npy ? make_npy(c, size_t(nrec), size_t(nt))
                    : Bytes(reinterpret_cast<const uint8_t*>(c), reinterpret_cast<const uint8_t*>(c + nobs));
      if (write_files_) write_file(p, b);
      out[p] = std::move(b);
    };
    if (sh) { emit("uy", 1, true); emit("vy", 1, false); }
    if (psv) {
      emit("ux", 0, true); emit("uz", 2, true);
      emit("vx", 0, false); emit("vz", 2, false);
      if (spin) { emit("ry", 1, true); emit("yi", 3, true); }
    }
    log_info("  -> traces saved to " + trace_dir);
  }
  if (snap_count > 0) {
    Bytes nf(4);
    std::memcpy(nf.data(), &snap_count, 4);
    out["snapshot/nframes"] = nf;
    for (auto& kv : snap_bufs) {
      const uint8_t* p = reinterpret_cast<const uint8_t*>(kv.second.data());
      out["snapshot/" + kv.first + ".f32"] = Bytes(p, p + kv.second.size() * 4);
    }
  }
  return out;
}

Vfs Solver::run_adjoint(const Vfs& vfs) {
  Vfs out;
  const bool sh = cfg_.sh;
  const int nt = int(cfg_.nt), nrec = this->nrec(), nsrc = this->nsrc();
  const uint32_t adj = cfg_.adj_interval;
  if (adj == 0) throw Error("adj_interval must be positive");
  const uint32_t nsa = cfg_.nt / adj;
  if (nsa == 0) throw Error("adj_interval (" + std::to_string(adj) + ") >= nt (" + std::to_string(nt) + ")");
  if (write_files_) mkdirs(cfg_.output);
  if (!cfg_.has_traces) throw Error("config [path] traces is required for the adjoint workflow");
  const std::string obs_dir = cfg_.traces;

  sim_->clear_kmu();
  std::vector<std::pair<int, int>> runs;
  if (cfg_.combine_sources) runs.push_back({-1, 0});
  else for (int s = 0; s < nsrc; ++s) runs.push_back({s, s});

  misfits_.clear();
  total_misfit_ = 0.0;
  std::vector<float> obs(size_t(5) * nrec * nt), adstf(size_t(nrec) * nt, 0.0f);
  const size_t nobs = size_t(nrec) * nt;
  for (size_t run = 0; run < runs.size(); ++run) {
    const int isrc = runs[run].first, ref_idx = runs[run].second;
    log_info("Adjoint: source " + std::to_string(run + 1) + "/" + std::to_string(runs.size()) + " (" +
             std::to_string(nt) + " steps, " + std::to_string(nsa) + " checkpoints)...");
    std::vector<float> ref;
    if (sh) {
      std::string p = path_join(obs_dir, "uy_" + fmt6(uint32_t(cfg_.combine_sources ? 0 : ref_idx)) + ".npy");
      Bytes b;
      try {
        b = lookup(vfs, p);
      } catch (const Error&) {
        throw Error("Cannot load observed traces " + p);
      }
      ref = parse_npy(b, p);
      if (ref.size() != nobs)
        throw Error("observed traces " + p + " hold " + std::to_string(ref.size()) + " samples, expected " +
                    std::to_string(nobs));
    }
    sim_->adjoint_forward(isrc, int(adj));
    double misfit = 0.0;
    if (sh) {
      sim_->download_traces(obs.data());
      misfit = waveform_misfit(obs.data() + nobs, ref.data(), nrec, nt, cfg_.dt, adstf.data());
    } else {
      std::fill(adstf.begin(), adstf.end(), 0.0f);
    }
    misfits_.push_back(misfit);
    total_misfit_ += misfit;
    char buf[96];
    std::snprintf(buf, sizeof buf, "Adjoint: source %zu misfit = %.6e", run + 1, misfit);
    log_info(buf);
    sim_->adjoint_backward(adstf.data(), int(adj));
  }
  {
    char buf[96];
    std::snprintf(buf, sizeof buf, "Adjoint: total misfit = %.6e", total_misfit_);
    log_info(buf);
  }
  sim_->smooth_kmu(cfg_.smooth);
  std::vector<float> kmu(size_t(grid_.nx) * grid_.nz);
  sim_->download_kmu(kmu.data());
  const std::string kp = path_join(cfg_.output, "proc000000_kmu.bin");
  const std::string gp = path_join(cfg_.output, "gradient_kmu.bin");
  const uint8_t* p = reinterpret_cast<const uint8_t*>(kmu.data());
  Bytes raw(p, p + kmu.size() * 4);
  Bytes with_header = make_model_bin(kmu);
  if (write_files_) {
    write_file(kp, raw);
    write_file(gp, with_header);
  }
  out[kp] = std::move(raw);
  out[gp] = std::move(with_header);
  log_info("Adjoint: gradient saved to " + kp);
  return out;
}

// ---- inversion ---------------------------------------------------------------
// Steepest descent in relative model units with a backtracking line search:
//   s_p  = m_p g_p / max over p and cells |m_p g_p|   (p: the inverted fields)
//   m_p <- m_p (1 - alpha s_p)                         (largest relative change alpha)
//   accept when J(m_new) <= J(m) + c1 sum g (m_new - m)  (Armijo, c1 = 1e-4),
//   else alpha <- alpha / 2, at most [inversion] line_search_trials times;
//   after an acceptance at the first trial the next step starts 1.5x larger.
// J is the L2 waveform misfit (l2_misfit) summed over the shots; its gradient
// is the exact discrete adjoint (Sim::forward_op / backward_op, checkpointed),
// mapped to vp, vs, rho and smoothed with the Gaussian of the reference's
// kernel smoothing (fd2d.wgsl:515-609).  A trial model that fails the
// stability check counts as a rejected trial.
Vfs Solver::run_inversion(const Vfs& vfs) {
  if (cfg_.spin || cfg_.sh == cfg_.psv) throw Error("the inversion workflow runs SH or PSV alone (no spin)");
  if (!cfg_.has_traces) throw Error("config [path] traces is required for the inversion workflow");
  const bool psv = cfg_.psv;
  const int nt = int(cfg_.nt), nrec = this->nrec(), nsrc = this->nsrc();
  const int ncomp = psv ? 2 : 1;
  const size_t npt = size_t(grid_.nx) * grid_.nz, nobs = size_t(nrec) * nt;
  std::vector<std::string> params;
  {
    std::stringstream ss(cfg_.inv_parameters);
    std::string t;
    while (std::getline(ss, t, ',')) {
      t = trim(t);
      if (t.empty()) continue;
      if (t != "vp" && t != "vs" && t != "rho") throw Error("[inversion] parameters: unknown field " + t);
      params.push_back(t);
    }
  }
  if (params.empty()) throw Error("[inversion] parameters lists no field");
  if (cfg_.inv_step <= 0.0f || cfg_.inv_max_step <= 0.0f) throw Error("[inversion] step and max_step must be > 0");

  // Shots as in run_adjoint, and their observed traces ([path] traces:
  // uy_NNNNNN.npy for SH; ux_ and uz_NNNNNN.npy for PSV, the forward
  // workflow's output names).
  std::vector<std::pair<int, int>> runs;
  if (cfg_.combine_sources) runs.push_back({-1, 0});
  else for (int s = 0; s < nsrc; ++s) runs.push_back({s, s});
  std::vector<std::vector<float>> obs(runs.size());
  for (size_t q = 0; q < runs.size(); ++q) {
    for (const char* c : psv ? std::vector<const char*>{"ux", "uz"} : std::vector<const char*>{"uy"}) {
      const std::string p = path_join(cfg_.traces, std::string(c) + "_" + fmt6(uint32_t(runs[q].second)) + ".npy");
      Bytes b;
      try {
        b = lookup(vfs, p);
      } catch (const Error&) {
        throw Error("Cannot load observed traces " + p);
      }
      std::vector<float> t = parse_npy(b, p);
      if (t.size() != nobs)
        throw Error("observed traces " + p + " hold " + std::to_string(t.size()) + " samples, expected " +
                    std::to_string(nobs));
      obs[q].insert(obs[q].end(), t.begin(), t.end());
    }
  }
  // The initial model, as read by the constructor.
  const std::string model_dir = cfg_.has_model_init ? cfg_.model_init : cfg_.model_true;
  std::map<std::string, std::vector<float>> model;
  Bytes x_bytes, z_bytes;
  for (const char* f : {"vp", "vs", "rho"}) {
    const std::string p = path_join(model_dir, std::string("proc000000_") + f + ".bin");
    model[f] = parse_model_bin(lookup(vfs, p), p);
    if (model[f].size() != npt) throw Error("a model file does not match the grid");
  }
  x_bytes = lookup(vfs, path_join(model_dir, "proc000000_x.bin"));
  z_bytes = lookup(vfs, path_join(model_dir, "proc000000_z.bin"));
  const float sigma = cfg_.inv_smooth >= 0.0f ? cfg_.inv_smooth : cfg_.smooth;
  const unsigned comp_mask = psv ? (1u << 0) | (1u << 2) : (1u << 1);
  std::vector<float> tr(size_t(5) * nobs), syn(size_t(ncomp) * nobs), adj(size_t(ncomp) * nobs);
  auto gather = [&]() {
    sim_->download_traces(tr.data(), comp_mask);
    if (psv) {
      std::copy(tr.begin(), tr.begin() + long(nobs), syn.begin());
      std::copy(tr.begin() + 2 * long(nobs), tr.begin() + 3 * long(nobs), syn.begin() + long(nobs));
    } else {
      std::copy(tr.begin() + long(nobs), tr.begin() + 2 * long(nobs), syn.begin());
    }
  };
  auto upload = [&](const std::map<std::string, std::vector<float>>& m) {
    sim_->upload_model(ModelField::VP, m.at("vp").data());
    sim_->upload_model(ModelField::VS, m.at("vs").data());
    sim_->upload_model(ModelField::RHO, m.at("rho").data());
    try {
      sim_->prepare_model();
    } catch (const std::invalid_argument& e) {
      log_info(std::string("Inversion: trial model rejected: ") + e.what());
      return false;
    }
    return true;
  };
  auto misfit = [&](const std::map<std::string, std::vector<float>>& m) {
    if (!upload(m)) return std::numeric_limits<double>::infinity();
    double J = 0.0;
    for (size_t q = 0; q < runs.size(); ++q) {
      sim_->run_forward(runs[q].first);
      gather();
      J += l2_misfit(syn.data(), obs[q].data(), ncomp * nrec, nt, cfg_.dt, nullptr);
    }
    return J;
  };
  std::map<std::string, std::vector<float>> grad;
  auto gradient = [&](const std::map<std::string, std::vector<float>>& m) {
    if (!upload(m)) throw Error("the current inversion model fails the stability check");
    sim_->gradient_clear();
    double J = 0.0;
    for (size_t q = 0; q < runs.size(); ++q) {
      sim_->forward_op(runs[q].first, 0);
      gather();
      J += l2_misfit(syn.data(), obs[q].data(), ncomp * nrec, nt, cfg_.dt, adj.data());
      sim_->backward_op(adj.data());
    }
    std::vector<float> gl(npt), gm(npt), gb(npt);
    sim_->download_gradient(0, gl.data());
    sim_->download_gradient(1, gm.data());
    sim_->download_gradient(2, gb.data());
    for (const char* f : {"vp", "vs", "rho"}) grad[f].assign(npt, 0.0f);
    velocity_gradients(gl.data(), gm.data(), gb.data(), m.at("vp").data(), m.at("vs").data(), m.at("rho").data(),
                       npt, grad["vp"].data(), grad["vs"].data(), grad["rho"].data());
    if (sigma > 0.0f)
      for (const std::string& p : params) sim_->smooth_field(grad[p].data(), sigma);
    return J;
  };

  inv_history_.clear();
  float alpha0 = std::min(cfg_.inv_step, cfg_.inv_max_step);
  for (uint32_t iter = 0; iter < cfg_.inv_iterations; ++iter) {
    const double J = gradient(model);
    double scale = 0.0;
    for (const std::string& p : params)
      for (size_t k = 0; k < npt; ++k) scale = std::max(scale, std::fabs(double(model[p][k]) * grad[p][k]));
    InversionStep rec{J, J, 0.0, 0, false};
    if (scale > 0.0) {
      float alpha = alpha0;
      for (uint32_t trial = 1; trial <= cfg_.inv_trials; ++trial) {
        auto cand = model;
        double slope = 0.0;
        for (const std::string& p : params)
          for (size_t k = 0; k < npt; ++k) {
            const double m0 = model[p][k], sp = m0 * grad[p][k] / scale;
            cand[p][k] = float(m0 * (1.0 - double(alpha) * sp));
            slope += double(grad[p][k]) * (double(cand[p][k]) - m0);
          }
        const double Jn = misfit(cand);
        rec.trials = int(trial);
        if (std::isfinite(Jn) && Jn <= J + 1e-4 * slope) {
          rec = InversionStep{J, Jn, double(alpha), int(trial), true};
          model = std::move(cand);
          alpha0 = std::min(alpha * (trial == 1 ? 1.5f : 1.0f), cfg_.inv_max_step);
          break;
        }
        alpha *= 0.5f;
        alpha0 = alpha;
      }
    }
    inv_history_.push_back(rec);
    char buf[160];
    std::snprintf(buf, sizeof buf, "Inversion: iteration %u misfit %.6e -> %.6e (step %.4g, %s after %d trial%s)",
                  iter + 1, rec.misfit, rec.new_misfit, rec.step, rec.accepted ? "accepted" : "rejected",
                  rec.trials, rec.trials == 1 ? "" : "s");
    log_info(buf);
    if (!rec.accepted) break;  // no descent found along the gradient: stop
  }
  upload(model);  // the simulation holds the final model

  Vfs out;
  if (write_files_) mkdirs(cfg_.output);
  auto emit = [&](const std::string& name, Bytes b) {
    const std::string p = path_join(cfg_.output, name);
    if (write_files_) write_file(p, b);
    out[p] = std::move(b);
  };
  for (const char* f : {"vp", "vs", "rho"}) emit(std::string("proc000000_") + f + ".bin", make_model_bin(model[f]));
  emit("proc000000_x.bin", x_bytes);
  emit("proc000000_z.bin", z_bytes);
  std::string log = "# iteration misfit new_misfit step trials accepted\n";
  for (size_t q = 0; q < inv_history_.size(); ++q) {
    char buf[160];
    const InversionStep& r = inv_history_[q];
    std::snprintf(buf, sizeof buf, "%zu %.9e %.9e %.6g %d %d\n", q + 1, r.misfit, r.new_misfit, r.step, r.trials,
                  int(r.accepted));
    log += buf;
  }
  emit("inversion_misfit.txt", Bytes(log.begin(), log.end()));
  log_info("Inversion: model saved to " + cfg_.output);
  return out;
}

}  // namespace seiswg
