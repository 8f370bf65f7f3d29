// C ABI of librp.so (declared in include/rp.h) plus the two on-disk formats
// next to the step: STL input (src/mesh.rs:125-143 via stl_io 0.7.0) and the
// legacy VTK output (src/vtk.rs:5-44).
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "engine.h"

struct rp_sim {
  rp::Engine* e;
};

namespace rp {

static thread_local std::string g_err;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
}

// ------------------------------------------------------------------- STL
// stl_io 0.7.0 (Cargo.lock) treats a file whose first line starts with
// "solid" as ASCII (facet normal / outer loop / 3 vertex / endloop / endfacet)
// and anything else as binary: 80-byte header, u32 triangle count, then
// 50-byte records of normal + three vertices (little-endian f32) + u16.
// Values are kept as f32, as the reference's Vec3 holds them.
static bool read_f32_le(const unsigned char* p, float* out) {
  uint32_t u = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
  std::memcpy(out, &u, 4);
  return true;
}

int load_stl(const char* path, std::vector<float>& v, std::vector<float>& n) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    set_error("cannot open STL file '%s'", path);
    return RP_E_IO;
  }
  std::vector<unsigned char> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  size_t first_nl = 0;
  while (first_nl < data.size() && data[first_nl] != '\n') ++first_nl;
  std::string line(data.begin(), data.begin() + first_nl);
  size_t s0 = 0;
  while (s0 < line.size() && std::isspace((unsigned char)line[s0])) ++s0;
  bool ascii = line.compare(s0, 5, "solid") == 0;
  if (ascii) {
    std::string text(data.begin(), data.end());
    std::istringstream in(text);
    std::string tok;
    in >> tok;  // solid
    std::getline(in, tok);
    std::vector<float> tv, tn;
    bool ok = true;
    while (in >> tok) {
      if (tok == "endsolid") break;
      if (tok != "facet") { ok = false; break; }
      std::string w;
      float nx, ny, nz;
      if (!(in >> w) || w != "normal" || !(in >> nx >> ny >> nz)) { ok = false; break; }
      if (!(in >> w) || w != "outer" || !(in >> w) || w != "loop") { ok = false; break; }
      for (int k = 0; k < 3 && ok; ++k) {
        float x, y, z;
        if (!(in >> w) || w != "vertex" || !(in >> x >> y >> z)) ok = false;
        else { tv.push_back(x); tv.push_back(y); tv.push_back(z); }
      }
      if (!ok) break;
      if (!(in >> w) || w != "endloop" || !(in >> w) || w != "endfacet") { ok = false; break; }
      tn.push_back(nx); tn.push_back(ny); tn.push_back(nz);
    }
    if (ok) {
      v.insert(v.end(), tv.begin(), tv.end());
      n.insert(n.end(), tn.begin(), tn.end());
      return RP_OK;
    }
    // a binary file whose header happens to start with "solid": fall through
  }
  if (data.size() < 84) {
    set_error("STL file '%s' is too short", path);
    return RP_E_IO;
  }
  uint32_t cnt = (uint32_t)data[80] | ((uint32_t)data[81] << 8) | ((uint32_t)data[82] << 16) | ((uint32_t)data[83] << 24);
  if (data.size() < 84 + 50ull * cnt) {
    set_error("binary STL file '%s' is truncated (%u triangles declared)", path, cnt);
    return RP_E_IO;
  }
  for (uint32_t t = 0; t < cnt; ++t) {
    const unsigned char* r = data.data() + 84 + 50ull * t;
    float q[12];
    for (int k = 0; k < 12; ++k) read_f32_le(r + 4 * k, &q[k]);
    n.push_back(q[0]); n.push_back(q[1]); n.push_back(q[2]);
    for (int k = 3; k < 12; ++k) v.push_back(q[k]);
  }
  return RP_OK;
}

// ------------------------------------------------------------------- VTK
// Rust's `{}` for f32: the shortest digit string that reads back to the same
// f32, written without an exponent.
static std::string rust_f32(float x) {
  if (std::isnan(x)) return "NaN";
  if (std::isinf(x)) return x > 0 ? "inf" : "-inf";
  if (x == 0.0f) return std::signbit(x) ? "-0" : "0";
  char buf[64];
  int prec = 1;
  for (; prec <= 9; ++prec) {
    snprintf(buf, sizeof(buf), "%.*e", prec - 1, (double)x);
    if (std::strtof(buf, nullptr) == x) break;
  }
  // buf = [-]d.ddde[+-]XX
  std::string s(buf);
  bool neg = s[0] == '-';
  if (neg) s = s.substr(1);
  size_t epos = s.find('e');
  int ex = std::atoi(s.c_str() + epos + 1);
  std::string dig;
  for (size_t i = 0; i < epos; ++i)
    if (s[i] != '.') dig.push_back(s[i]);
  while (dig.size() > 1 && dig.back() == '0') dig.pop_back();
  std::string out;
  int point = ex + 1;  // digits before the decimal point
  if (point <= 0) {
    out = "0." + std::string(-point, '0') + dig;
  } else if ((size_t)point >= dig.size()) {
    out = dig + std::string(point - dig.size(), '0');
  } else {
    out = dig.substr(0, point) + "." + dig.substr(point);
  }
  return neg ? "-" + out : out;
}

int Engine::write_vtk(const char* path) {
  if (!host_valid_) {
    int r = download();
    if (r != RP_OK) return r;
  }
  FILE* f = std::fopen(path, "w");
  if (!f) {
    set_error("cannot create '%s'", path);
    return RP_E_IO;
  }
  const size_t n = hp_.size();
  std::fprintf(f, "# vtk DataFile Version 3.0\nDEM Simulation Data\nASCII\nDATASET POLYDATA\n");
  std::fprintf(f, "POINTS %zu float\n", n);
  for (const HostParticle& p : hp_)
    std::fprintf(f, "%s %s %s\n", rust_f32((float)p.x[0]).c_str(), rust_f32((float)p.x[1]).c_str(),
                 rust_f32((float)p.x[2]).c_str());
  std::fprintf(f, "POINT_DATA %zu\nVECTORS velocity float\n", n);
  for (const HostParticle& p : hp_)
    std::fprintf(f, "%s %s %s\n", rust_f32((float)p.v[0]).c_str(), rust_f32((float)p.v[1]).c_str(),
                 rust_f32((float)p.v[2]).c_str());
  std::fprintf(f, "SCALARS radius float 1\nLOOKUP_TABLE default\n");
  for (const HostParticle& p : hp_) std::fprintf(f, "%s\n", rust_f32((float)p.r).c_str());
  std::fprintf(f, "SCALARS id int 1\nLOOKUP_TABLE default\n");
  for (size_t i = 0; i < n; ++i) std::fprintf(f, "%zu\n", i);
  bool ok = std::ferror(f) == 0;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    set_error("write to '%s' failed", path);
    return RP_E_IO;
  }
  return RP_OK;
}

}  // namespace rp

using rp::set_error;

#define SIM_OR_FAIL(s)                 \
  do {                                 \
    if (!(s) || !(s)->e) {             \
      set_error("null simulation handle"); \
      return RP_E_INVALID_ARG;         \
    }                                  \
  } while (0)

static bool finite3(const double* a) { return std::isfinite(a[0]) && std::isfinite(a[1]) && std::isfinite(a[2]); }

static int check_material(double E, double nu, double mu, double e) {
  if (!(E > 0.0) || !std::isfinite(nu) || !(mu >= 0.0) || !(e >= 0.0)) {
    set_error("material needs E > 0, finite nu, friction >= 0 and restitution >= 0");
    return RP_E_INVALID_ARG;
  }
  return RP_OK;
}

extern "C" {

rp_sim* rp_create(double dt, const double min_xyz[3], const double max_xyz[3], size_t particle_capacity) {
  if (!min_xyz || !max_xyz || !(dt > 0.0) || !finite3(min_xyz) || !finite3(max_xyz)) {
    set_error("rp_create needs dt > 0 and finite bounds");
    return nullptr;
  }
  rp_sim* s = new (std::nothrow) rp_sim;
  if (!s) return nullptr;
  s->e = new (std::nothrow) rp::Engine(dt, min_xyz, max_xyz, particle_capacity);
  if (!s->e) {
    delete s;
    return nullptr;
  }
  return s;
}

void rp_destroy(rp_sim* s) {
  if (!s) return;
  delete s->e;
  delete s;
}

int rp_add_particle(rp_sim* s, double x, double y, double z, double radius, double mass, int fixed) {
  SIM_OR_FAIL(s);
  double p[3] = {x, y, z};
  return s->e->add_particle(p, radius, mass, fixed);
}

int rp_add_particles(rp_sim* s, size_t n, const double* xyz, const double* radius, const double* mass,
                     const uint8_t* fixed) {
  SIM_OR_FAIL(s);
  if (n && (!xyz || !radius || !mass)) {
    set_error("rp_add_particles: null array");
    return RP_E_INVALID_ARG;
  }
  return s->e->add_particles(n, xyz, radius, mass, fixed);
}

int rp_add_mesh_stl(rp_sim* s, const char* path) {
  SIM_OR_FAIL(s);
  if (!path) {
    set_error("null path");
    return RP_E_IO;
  }
  std::vector<float> v, n;
  int r = rp::load_stl(path, v, n);
  if (r != RP_OK) return r;
  return s->e->add_triangles(v.size() / 9, v.data(), n.data());
}

int rp_add_mesh_triangles(rp_sim* s, size_t n_triangles, const float* vertices, const float* normals) {
  SIM_OR_FAIL(s);
  if (n_triangles && !vertices) {
    set_error("null vertex array");
    return RP_E_INVALID_ARG;
  }
  return s->e->add_triangles(n_triangles, vertices, normals);
}

int rp_add_mesh_triangles_group(rp_sim* s, size_t n_triangles, const float* vertices, const float* normals,
                                uint32_t group) {
  SIM_OR_FAIL(s);
  if (n_triangles && !vertices) {
    set_error("null vertex array");
    return RP_E_INVALID_ARG;
  }
  if (group != RP_GROUP_ALL && group >= (1u << 24)) {
    set_error("group id %u too large (at most 2^24 - 1)", group);
    return RP_E_INVALID_ARG;
  }
  return s->e->add_triangles(n_triangles, vertices, normals, group);
}

int rp_add_mesh_triangles_moving(rp_sim* s, size_t n_triangles, const float* vertices, const float* normals,
                                 uint32_t group, const double center[3], const double omega[3],
                                 const double velocity[3]) {
  SIM_OR_FAIL(s);
  if (n_triangles && !vertices) {
    set_error("null vertex array");
    return RP_E_INVALID_ARG;
  }
  if (!center || !omega || !velocity || !finite3(center) || !finite3(omega) || !finite3(velocity)) {
    set_error("moving wall needs finite center, omega and velocity");
    return RP_E_INVALID_ARG;
  }
  if (group != RP_GROUP_ALL && group >= (1u << 24)) {
    set_error("group id %u too large (at most 2^24 - 1)", group);
    return RP_E_INVALID_ARG;
  }
  rp::WallMotion m;
  for (int k = 0; k < 3; ++k) {
    m.c[k] = center[k];
    m.w[k] = omega[k];
    m.v[k] = velocity[k];
  }
  return s->e->add_triangles(n_triangles, vertices, normals, group, &m);
}

int rp_set_particle_groups(rp_sim* s, size_t n, const uint32_t* groups) {
  SIM_OR_FAIL(s);
  if (n && !groups) {
    set_error("null group array");
    return RP_E_INVALID_ARG;
  }
  return s->e->set_particle_groups(n, groups);
}

int rp_get_particle_groups(rp_sim* s, size_t n, uint32_t* groups) {
  SIM_OR_FAIL(s);
  if (n && !groups) {
    set_error("null group array");
    return RP_E_INVALID_ARG;
  }
  return s->e->get_particle_groups(n, groups);
}

int rp_set_group_material(rp_sim* s, uint32_t group, double E, double nu, double rho, double mu, double e,
                          double gamma) {
  SIM_OR_FAIL(s);
  int r = check_material(E, nu, mu, e);
  if (r != RP_OK) return r;
  return s->e->set_group_material(group, rp::Material{E, nu, rho, mu, e, gamma});
}

int rp_set_particle_material(rp_sim* s, double E, double nu, double rho, double mu, double e, double gamma) {
  SIM_OR_FAIL(s);
  int r = check_material(E, nu, mu, e);
  if (r != RP_OK) return r;
  s->e->pm = rp::Material{E, nu, rho, mu, e, gamma};
  s->e->config_changed();
  return RP_OK;
}

int rp_set_wall_material(rp_sim* s, double E, double nu, double rho, double mu, double e, double gamma) {
  SIM_OR_FAIL(s);
  int r = check_material(E, nu, mu, e);
  if (r != RP_OK) return r;
  s->e->wm = rp::Material{E, nu, rho, mu, e, gamma};
  s->e->config_changed();
  return RP_OK;
}

int rp_set_contact_models(rp_sim* s, int normal_model, int tangential_model) {
  SIM_OR_FAIL(s);
  if (normal_model < 0 || normal_model > 4 || tangential_model < 0 || tangential_model > 2) {
    set_error("Invalid contact model id");
    return RP_E_INVALID_ARG;
  }
  s->e->nmodel = normal_model;
  s->e->tmodel = tangential_model;
  s->e->config_changed();
  return RP_OK;
}

int rp_parse_contact_models(const char* normal, const char* tangential, int* nm, int* tm) {
  if (!normal || !tangential || !nm || !tm) {
    set_error("null argument");
    return RP_E_INVALID_ARG;
  }
  auto lower = [](const char* c) {
    std::string s(c);
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
  };
  std::string a = lower(normal), b = lower(tangential);
  int n = -1, t = -1;
  if (a == "hertz" || a == "hertzian") n = RP_NORMAL_HERTZ;
  else if (a == "linear" || a == "spring_dashpot") n = RP_NORMAL_LINEAR;
  else if (a == "hysteretic") n = RP_NORMAL_HYSTERETIC;
  else if (a == "jkr") n = RP_NORMAL_JKR;
  else if (a == "sjkr" || a == "simplified_jkr") n = RP_NORMAL_SJKR;
  if (n < 0) {
    set_error("Invalid normal force model");
    return RP_E_INVALID_ARG;
  }
  if (b == "mindlin") t = RP_TANGENTIAL_MINDLIN;
  else if (b == "coulomb") t = RP_TANGENTIAL_COULOMB;
  else if (b == "linear" || b == "spring_coulomb") t = RP_TANGENTIAL_LINEAR_SPRING;
  if (t < 0) {
    set_error("Invalid tangential force model");
    return RP_E_INVALID_ARG;
  }
  *nm = n;
  *tm = t;
  return RP_OK;
}

int rp_set_periodic(rp_sim* s, int x, int y, int z) {
  SIM_OR_FAIL(s);
  s->e->periodic[0] = x != 0;
  s->e->periodic[1] = y != 0;
  s->e->periodic[2] = z != 0;
  s->e->config_changed();
  return RP_OK;
}

int rp_enable_gpu(rp_sim* s, int device) {
  SIM_OR_FAIL(s);
  return s->e->enable_gpu(device);
}

int rp_step(rp_sim* s, uint64_t n) {
  SIM_OR_FAIL(s);
  return s->e->step(n);
}

int rp_run(rp_sim* s, double duration) {
  SIM_OR_FAIL(s);
  // src/lib.rs:356: (duration / dt).ceil() as usize, in f32
  float q = (float)duration / (float)s->e->dt;
  float c = std::ceil(q);
  uint64_t steps = (!(c > 0.0f)) ? 0 : (c >= 1.8e19f ? UINT64_MAX : (uint64_t)c);
  return s->e->step(steps);
}

size_t rp_particle_count(rp_sim* s) {
  if (!s || !s->e) return 0;
  return s->e->count();
}

int rp_get_particle_position(rp_sim* s, size_t id, double out[3]) {
  SIM_OR_FAIL(s);
  return s->e->get_vec(id, 0, out);
}
int rp_get_particle_velocity(rp_sim* s, size_t id, double out[3]) {
  SIM_OR_FAIL(s);
  return s->e->get_vec(id, 1, out);
}
int rp_get_particle_angular_velocity(rp_sim* s, size_t id, double out[3]) {
  SIM_OR_FAIL(s);
  return s->e->get_vec(id, 2, out);
}
int rp_set_particle_velocity(rp_sim* s, size_t id, double vx, double vy, double vz) {
  SIM_OR_FAIL(s);
  double v[3] = {vx, vy, vz};
  return s->e->set_vec(id, 1, v);
}
int rp_set_particle_angular_velocity(rp_sim* s, size_t id, double wx, double wy, double wz) {
  SIM_OR_FAIL(s);
  double v[3] = {wx, wy, wz};
  return s->e->set_vec(id, 2, v);
}

int rp_write_vtk(rp_sim* s, const char* path) {
  SIM_OR_FAIL(s);
  if (!path) {
    set_error("null path");
    return RP_E_IO;
  }
  return s->e->write_vtk(path);
}

// Both directions move n_particles entries per array: the caller declares the
// length of its arrays there, and a length other than the live particle count
// is rejected before any array is touched.
int rp_read_state(rp_sim* s, rp_state* out) {
  SIM_OR_FAIL(s);
  if (!out) {
    set_error("null state");
    return RP_E_INVALID_ARG;
  }
  const size_t n = s->e->count();
  if (out->n_particles != n) {
    set_error("state arrays hold %zu particles, the simulation has %zu", out->n_particles, n);
    return RP_E_INVALID_ARG;
  }
  return s->e->read_state(out);
}
int rp_write_state(rp_sim* s, const rp_state* in) {
  SIM_OR_FAIL(s);
  if (!in) {
    set_error("null state");
    return RP_E_INVALID_ARG;
  }
  const size_t n = s->e->count();
  if (in->n_particles != n) {
    set_error("state arrays hold %zu particles, the simulation has %zu", in->n_particles, n);
    return RP_E_INVALID_ARG;
  }
  return s->e->write_state(in);
}

int rp_set_precision(rp_sim* s, int precision) {
  SIM_OR_FAIL(s);
  if (precision != RP_PREC_FP64 && precision != RP_PREC_MIXED) {
    set_error("unknown precision mode %d", precision);
    return RP_E_INVALID_ARG;
  }
  s->e->prec = precision;
  s->e->config_changed();
  return RP_OK;
}
int rp_set_interaction_mode(rp_sim* s, int mode) {
  SIM_OR_FAIL(s);
  if (mode != RP_MODE_PARITY && mode != RP_MODE_PHYSICAL) {
    set_error("unknown interaction mode %d", mode);
    return RP_E_INVALID_ARG;
  }
  s->e->mode = mode;
  s->e->config_changed();
  return RP_OK;
}
int rp_set_gravity(rp_sim* s, double gx, double gy, double gz) {
  SIM_OR_FAIL(s);
  s->e->gravity[0] = gx;
  s->e->gravity[1] = gy;
  s->e->gravity[2] = gz;
  s->e->config_changed();
  return RP_OK;
}
int rp_set_reference_cell_size(rp_sim* s, double h) {
  SIM_OR_FAIL(s);
  if (!(h > 0.0)) {
    set_error("cell size must be positive");
    return RP_E_INVALID_ARG;
  }
  s->e->href = h;
  s->e->config_changed();
  return RP_OK;
}
int rp_set_skin(rp_sim* s, double skin) {
  SIM_OR_FAIL(s);
  s->e->skin_user = skin;
  s->e->config_changed();
  return RP_OK;
}

int rp_set_neighbor_capacity(rp_sim* s, int capacity) {
  SIM_OR_FAIL(s);
  if (capacity < 1 || capacity > 4096) {
    set_error("neighbour capacity must be in [1, 4096]");
    return RP_E_INVALID_ARG;
  }
  s->e->set_capacity(capacity);
  return RP_OK;
}

int rp_set_force_path(rp_sim* s, int path) {
  SIM_OR_FAIL(s);
  if (path != 0 && path != 1) {
    set_error("force path must be 0 or 1");
    return RP_E_INVALID_ARG;
  }
  s->e->force_path = path;
  s->e->config_changed();
  return RP_OK;
}

int rp_set_device_loop(rp_sim* s, int enable) {
  SIM_OR_FAIL(s);
  s->e->use_graph_ = enable != 0;
  return RP_OK;
}

static int g_threads_set = 0;
int rp_set_threads(int n) {
  // The reference sizes rayon's global pool once (src/lib.rs:15-22); a second
  // call fails the same way. Host threads only serve I/O here.
  if (n < 0) {
    set_error("thread count must be >= 0");
    return RP_E_INVALID_ARG;
  }
  if (g_threads_set) {
    set_error("Failed to set num threads: The global thread pool has already been initialized.");
    return RP_E_CUDA;
  }
  g_threads_set = 1;
  return RP_OK;
}

int rp_get_stats(rp_sim* s, rp_stats* out) {
  SIM_OR_FAIL(s);
  if (!out) {
    set_error("null stats");
    return RP_E_INVALID_ARG;
  }
  return s->e->stats(out);
}

int rp_set_profiling(rp_sim* s, int enable) {
  SIM_OR_FAIL(s);
  s->e->profiling = enable != 0;
  return RP_OK;
}

const char* rp_last_error(void) { return rp::g_err.c_str(); }
const char* rp_version(void) { return "rusty_particles_gb300 0.1.0 (sm_103a)"; }

int rp_set_debug(rp_sim* s, int enable) {
  SIM_OR_FAIL(s);
  s->e->debug = enable != 0;
  s->e->config_changed();
  return RP_OK;
}
int rp_debug_last_forces(rp_sim* s, double* force, double* torque) {
  SIM_OR_FAIL(s);
  if (!force || !torque) {
    set_error("null output");
    return RP_E_INVALID_ARG;
  }
  return s->e->debug_forces(force, torque);
}
int rp_debug_contact_pairs(rp_sim* s, int64_t* pi, int64_t* pj, int32_t* visits, size_t capacity, size_t* n) {
  SIM_OR_FAIL(s);
  if (!n) {
    set_error("null count");
    return RP_E_INVALID_ARG;
  }
  return s->e->debug_pairs(pi, pj, visits, capacity, n);
}
int rp_debug_reference_grid(rp_sim* s, double h, int64_t* cell_of, int64_t* order, size_t* n_order, int32_t dims[3]) {
  SIM_OR_FAIL(s);
  if (!cell_of || !order || !n_order || !dims || !(h > 0.0)) {
    set_error("bad argument");
    return RP_E_INVALID_ARG;
  }
  return s->e->debug_reference_grid(h, cell_of, order, n_order, dims);
}

int rp_bed_statistics(rp_sim* s, double out[3]) {
  SIM_OR_FAIL(s);
  if (!out) {
    set_error("null output");
    return RP_E_INVALID_ARG;
  }
  return s->e->bed_statistics(out);
}

int rp_debug_triangle_grid(rp_sim* s, int32_t dims[3], double lo_cell[4], uint32_t* start, size_t start_cap,
                           uint32_t* items, size_t items_cap, size_t* n_start, size_t* n_items) {
  SIM_OR_FAIL(s);
  if (!dims || !lo_cell || !n_start || !n_items) {
    set_error("bad argument");
    return RP_E_INVALID_ARG;
  }
  return s->e->debug_triangle_grid(dims, lo_cell, start, start_cap, items, items_cap, n_start, n_items);
}

int rp_autotune(rp_sim* s, rp_tune_report* report) {
  SIM_OR_FAIL(s);
  return s->e->autotune(report);
}

int rp_set_launch_shape(rp_sim* s, int bs_filter, int bs_force, int bs_accum, int grid_cap) {
  SIM_OR_FAIL(s);
  const int b[3] = {bs_filter, bs_force, bs_accum};
  for (int k = 0; k < 3; ++k)
    if (b[k] != 0 && (b[k] < 32 || b[k] > 256 || b[k] % 32 != 0)) {
      set_error("block sizes must be multiples of 32 in [32, 256] (0 = default)");
      return RP_E_INVALID_ARG;
    }
  if (grid_cap < 0) {
    set_error("grid cap must be >= 0");
    return RP_E_INVALID_ARG;
  }
  s->e->bs_filter = bs_filter;
  s->e->bs_force = bs_force;
  s->e->bs_accum = bs_accum;
  s->e->grid_cap = grid_cap;
  s->e->config_changed();
  return RP_OK;
}

// ---------------------------------------------------------- learned JKR
int rp_jkr_train(rp_sim* s, const rp_jkr_train_options* options, rp_jkr_train_report* report) {
  SIM_OR_FAIL(s);
  return s->e->jkr_train(options, report);
}
int rp_set_jkr_solver(rp_sim* s, int solver) {
  SIM_OR_FAIL(s);
  if (solver != RP_JKR_NEWTON && solver != RP_JKR_LEARNED && solver != RP_JKR_CERTIFIED) {
    set_error("unknown JKR solver %d", solver);
    return RP_E_INVALID_ARG;
  }
  if (solver == RP_JKR_LEARNED && !s->e->jkr_has_network()) {
    set_error("the learned JKR solver needs a network (rp_jkr_train or rp_jkr_set_network)");
    return RP_E_INVALID_ARG;
  }
  s->e->jkr_solver = solver;
  s->e->config_changed();
  return RP_OK;
}
int rp_jkr_get_network(rp_sim* s, float* params, float* norm, float* domain) {
  SIM_OR_FAIL(s);
  return s->e->jkr_get_network(params, norm, domain);
}
int rp_jkr_set_network(rp_sim* s, const float* params, const float* norm, const float* domain) {
  SIM_OR_FAIL(s);
  if (!params || !norm || !domain) {
    set_error("null network buffer");
    return RP_E_INVALID_ARG;
  }
  return s->e->jkr_set_network(params, norm, domain);
}
int rp_jkr_counters(rp_sim* s, uint64_t out[6]) {
  SIM_OR_FAIL(s);
  if (!out) {
    set_error("null output");
    return RP_E_INVALID_ARG;
  }
  return s->e->jkr_counters(out);
}

}  // extern "C"

namespace {

int need_device() {
  int cnt = 0;
  cudaError_t e = cudaGetDeviceCount(&cnt);
  if (e != cudaSuccess || cnt == 0) {
    rp::set_error("no usable CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0");
    return RP_E_CUDA;
  }
  return RP_OK;
}

// Device copies of host arrays for the standalone network entry points.
struct DevBufs {
  std::vector<void*> ptrs;
  ~DevBufs() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  T* get(size_t n, const T* src) {
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    if (src && n && cudaMemcpy(p, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return (T*)p;
  }
};

int cuda_fail(const char* what) {
  rp::set_error("%s failed: %s", what, cudaGetErrorString(cudaGetLastError()));
  return RP_E_CUDA;
}

}  // namespace

extern "C" {

int rp_mlp_loss_grad(const float* params, const float* features, const float* targets, const float* weights, size_t n,
                     int qat, float* grad, double* loss) {
  if (!params || !features || !targets || !weights || !grad || !loss || n < 64 || (n & (n - 1)) != 0) {
    set_error("rp_mlp_loss_grad needs all buffers and n a power of two >= 64");
    return RP_E_INVALID_ARG;
  }
  int r = need_device();
  if (r) return r;
  DevBufs B;
  float* p = B.get(rp::MLP_NPARAM, params);
  float* f = B.get(4 * n, features);
  float* t = B.get(n, targets);
  float* w = B.get(n, weights);
  float* g = B.get<float>(rp::MLP_NPARAM, nullptr);
  if (!p || !f || !t || !w || !g) return cuda_fail("device allocation");
  if (rp::mlp_loss_grad(p, f, t, w, n, qat, g, loss, 0) != 0) return cuda_fail("network gradient");
  if (cudaMemcpy(grad, g, sizeof(float) * rp::MLP_NPARAM, cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_fail("gradient copy");
  return RP_OK;
}

int rp_mlp_infer(const float* params, const float* features, size_t n, float* out) {
  if (!params || !features || !out) {
    set_error("null buffer");
    return RP_E_INVALID_ARG;
  }
  int r = need_device();
  if (r) return r;
  rp::MlpInfer h;
  const float norm[10] = {0, 0, 0, 0, 1, 1, 1, 1, 0, 1};
  rp::mlp_make_infer(params, norm, &h);
  DevBufs B;
  rp::MlpInfer* m = B.get(1, &h);
  float* f = B.get(4 * n, features);
  float* o = B.get<float>(n, nullptr);
  if (!m || !f || !o) return cuda_fail("device allocation");
  if (rp::mlp_infer_rows(m, f, n, o, 0) != 0) return cuda_fail("network inference");
  if (n && cudaMemcpy(out, o, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return cuda_fail("output copy");
  return RP_OK;
}

int rp_jkr_samples(const double domain[8], uint64_t seed, size_t n, float* features, float* targets, float* weights,
                   double* a_ref, int32_t* iters, double* inputs) {
  if (!domain || !features || !targets || !weights) {
    set_error("null buffer");
    return RP_E_INVALID_ARG;
  }
  for (int k = 0; k < 6; ++k)
    if (!(domain[k] > 0.0)) {
      set_error("domain radius, modulus and surface-energy bounds must be positive");
      return RP_E_INVALID_ARG;
    }
  int r = need_device();
  if (r) return r;
  rp::JkrDomain D{domain[0], domain[1], domain[2], domain[3], domain[4], domain[5], domain[6], domain[7]};
  DevBufs B;
  float* f = B.get<float>(4 * n, nullptr);
  float* t = B.get<float>(n, nullptr);
  float* w = B.get<float>(n, nullptr);
  double* a = a_ref ? B.get<double>(n, nullptr) : nullptr;
  int32_t* it = iters ? B.get<int32_t>(n, nullptr) : nullptr;
  double* in = inputs ? B.get<double>(4 * n, nullptr) : nullptr;
  if (!f || !t || !w || (a_ref && !a) || (iters && !it) || (inputs && !in)) return cuda_fail("device allocation");
  if (rp::jkr_generate_samples(D, seed, n, f, t, w, a, it, in, 0) != 0) return cuda_fail("sample generation");
  if (n) {
    if (cudaMemcpy(features, f, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(targets, t, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(weights, w, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        (a_ref && cudaMemcpy(a_ref, a, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (iters && cudaMemcpy(iters, it, sizeof(int32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess) ||
        (inputs && cudaMemcpy(inputs, in, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost) != cudaSuccess))
      return cuda_fail("sample copy");
  }
  return RP_OK;
}

}  // extern "C"
