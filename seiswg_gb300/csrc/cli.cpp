// cli.cpp -- `seiswg <config.ini>`, the command-line entry of the reference
// (src/main.rs:33-99): load the config, pre-load the model directory,
// sources, stations and observed traces into a VFS, then run the workflow:
// forward, adjoint, or inversion (which the reference rejects as not yet
// implemented, main.rs:93-94).
#include <dirent.h>
#include <sys/stat.h>

#include <cstdio>
#include <fstream>
#include <string>

#include "../../include/seiswg.h"

namespace {

bool is_dir(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

bool is_file(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

void add_file(seiswg_vfs* vfs, const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  std::string bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  seiswg_vfs_insert(vfs, path.c_str(), bytes.data(), bytes.size());
}

// main.rs:17-31: every file under `dir`, keyed by its path.
void load_dir(seiswg_vfs* vfs, const std::string& dir) {
  DIR* d = ::opendir(dir.c_str());
  if (!d) return;
  while (struct dirent* e = ::readdir(d)) {
    std::string n = e->d_name;
    if (n == "." || n == "..") continue;
    std::string p = dir + "/" + n;
    if (is_dir(p)) load_dir(vfs, p);
    else if (is_file(p)) add_file(vfs, p);
  }
  ::closedir(d);
}

int die(const char* what) {
  std::fprintf(stderr, "Error: %s: %s\n", what, seiswg_last_error());
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "Usage: %s <config.ini>\n", argv[0]);
    return 1;
  }
  seiswg_config* cfg = nullptr;
  if (seiswg_config_load(argv[1], &cfg) != SEISWG_OK) return die("Failed to load config");
  char buf[4096];
  seiswg_vfs* vfs = seiswg_vfs_new();
  if (seiswg_config_get(cfg, "path.model_init", buf, sizeof buf) == SEISWG_OK ||
      seiswg_config_get(cfg, "path.model_true", buf, sizeof buf) == SEISWG_OK)
    load_dir(vfs, buf);
  if (seiswg_config_get(cfg, "path.model_true", buf, sizeof buf) == SEISWG_OK) load_dir(vfs, buf);
  if (seiswg_config_get(cfg, "path.sources", buf, sizeof buf) == SEISWG_OK && is_file(buf)) add_file(vfs, buf);
  if (seiswg_config_get(cfg, "path.stations", buf, sizeof buf) == SEISWG_OK && is_file(buf)) add_file(vfs, buf);
  if (seiswg_config_get(cfg, "path.traces", buf, sizeof buf) == SEISWG_OK) load_dir(vfs, buf);

  seiswg_solver* s = nullptr;
  if (seiswg_solver_new(cfg, vfs, &s) != SEISWG_OK) return die("Failed to initialise solver");
  char wf[64];
  seiswg_config_get(cfg, "workflow", wf, sizeof wf);
  std::string workflow = wf;
  int rc = 0;
  if (workflow == "forward") {
    if (seiswg_solver_run_forward(s, nullptr) != SEISWG_OK) rc = die("forward");
  } else if (workflow == "adjoint") {
    if (seiswg_solver_run_adjoint(s, vfs, nullptr) != SEISWG_OK) rc = die("adjoint");
  } else if (workflow == "inversion") {
    if (seiswg_solver_run_inversion(s, vfs, nullptr) != SEISWG_OK) rc = die("inversion");
  } else {
    std::fprintf(stderr, "Error: Workflow '%s' is not yet implemented in seiswg\n", workflow.c_str());
    rc = 1;
  }
  if (rc == 0) std::fprintf(stderr, "[seiswg] Done.\n");
  seiswg_solver_free(s);
  seiswg_vfs_free(vfs);
  seiswg_config_free(cfg);
  return rc;
}
