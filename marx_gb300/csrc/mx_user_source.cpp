// USER sources: a plug-in shared object with user_open_source,
// user_create_ray, user_close_source and optionally user_start_iteration,
// loaded and driven as marx_select_user_source, open_source, create_photons
// and close_source do (marx/libsrc/s-user.c:57-300).  Host code: the
// plug-in's rays come one call at a time from the host, as in the
// reference; the photons it fills are then traced like any other.
#include <dlfcn.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/marx_gb300.h"

struct mx_user_source {
  void *handle = nullptr;
  int (*open_fn)(char **, int, double, double, double, double) = nullptr;
  void (*close_fn)(void) = nullptr;
  int (*ray_fn)(double *, double *, double *, double *, double *) = nullptr;
  int (*start_fn)(void) = nullptr;
  std::string args;            // UserSourceArgs, split in place into argv
  std::vector<char *> argv;
};

namespace {

thread_local std::string g_user_err;

bool white(char c) { return c == ' ' || c == '\t' || c == '\n'; }

// cmdline_to_argv_argc (s-user.c:97-140): words split at blanks, tabs and
// newlines, written over the string; argv ends with NULL.
void split_args(std::string &cmd, std::vector<char *> &argv) {
  argv.clear();
  char *p = &cmd[0];
  while (white(*p)) p++;
  while (*p) {
    argv.push_back(p);
    while (*p && !white(*p)) p++;
    if (*p) *p++ = 0;
    while (white(*p)) p++;
  }
  argv.push_back(nullptr);
}

void *sym(mx_user_source *s, const char *name, bool required) {
  void *f = dlsym(s->handle, name);
  if (!f && required) g_user_err = std::string("Unable to find symbol ") + name + " in the user source";
  return f;
}

}  // namespace

extern "C" {

mx_user_source *mx_user_source_open(const char *file, const char *args, double geometric_area, const double p[3]) {
  if (!file || !p) { g_user_err = "mx_user_source_open: null argument"; return nullptr; }
  auto *s = new mx_user_source;
  s->handle = dlopen(file, RTLD_LAZY);
  if (!s->handle) {
    const char *e = dlerror();
    g_user_err = std::string("Error linking to ") + file + "\nReason: " + (e ? e : "UNKNOWN");
    delete s;
    return nullptr;
  }
  s->open_fn = (int (*)(char **, int, double, double, double, double)) sym(s, "user_open_source", true);
  s->close_fn = (void (*)(void)) sym(s, "user_close_source", true);
  s->ray_fn = (int (*)(double *, double *, double *, double *, double *)) sym(s, "user_create_ray", true);
  s->start_fn = (int (*)(void)) sym(s, "user_start_iteration", false);
  if (!s->open_fn || !s->close_fn || !s->ray_fn) {
    dlclose(s->handle);
    delete s;
    return nullptr;
  }
  s->args = args ? args : "";
  split_args(s->args, s->argv);
  if (-1 == s->open_fn(s->argv.data(), (int) s->argv.size() - 1, geometric_area, p[0], p[1], p[2])) {
    g_user_err = "user_open_source failed";
    dlclose(s->handle);
    delete s;
    return nullptr;
  }
  return s;
}

int mx_user_source_create(mx_user_source *s, const mx_photons *h, uint32_t n, uint32_t *n_created, int *times_set) {
  if (!s || !h || !n_created || !h->energy || !h->p) { g_user_err = "mx_user_source_create: null argument"; return MX_EINVAL; }
  const size_t st = h->stride ? h->stride : h->n;
  if (n > h->n || st < h->n) { g_user_err = "mx_user_source_create: n beyond the list"; return MX_EINVAL; }
  *n_created = 0;
  if (times_set) *times_set = 0;
  if (s->start_fn && -1 == s->start_fn()) return MX_OK;
  double t = -1.0, last_time = 0.0;
  uint32_t i = 0;
  for (; i < n; i++) {
    const double drawn = h->energy[i];
    double energy = drawn, p1, p2, p3;
    if (-1 == s->ray_fn(&t, &energy, &p1, &p2, &p3)) break;
    if (h->flags) h->flags[i] = 0;
    h->p[i] = p1; h->p[st + i] = p2; h->p[2 * st + i] = p3;
    if (t >= 0.0) {
      last_time += t;
      if (h->arrival_time) h->arrival_time[i] = last_time;
    }
    if (energy < 0.0) energy = drawn;
    h->energy[i] = energy;
  }
  *n_created = i;
  if (times_set) *times_set = t >= 0.0;
  return MX_OK;
}

void mx_user_source_close(mx_user_source *s) {
  if (!s) return;
  if (s->close_fn) s->close_fn();
  if (s->handle) dlclose(s->handle);
  delete s;
}

const char *mx_user_source_error(void) { return g_user_err.c_str(); }

}  // extern "C"
