// cube_main -- CUBE's driver loop as a compiled caller of the C ABI.
//
// The reference's program main (CUBEnu/work/main/main.f90:88-145) calls, per
// step, timestep, update_x, buffer_grid, buffer_x, ext_pp_force,
// particle_mesh and buffer_v, and on a checkpoint step drifts the half step
// (dt_old = 0, update_x) before writing the checkpoint.  This program keeps
// that loop and its host-side scalar logic -- timestep and expansion
// (timestep.f90:1-92, 133-177) and the dt constraints of pm.f90:391-407 and
// ext_pp_force.f90:141 -- in C++, and every per-step subroutine body is a call
// into libcube_gb300.so through include/cube_gpu.h.  It is what a Fortran
// driver does through iso_c_binding, written for a machine without a Fortran
// compiler.
//
// Usage:
//   cube_main --out DIR [--nc 32] [--nnt 1] [--np-nc 2] [--box 200] [--pp 0]
//             [--rsoft 0.1] [--z-init 49] [--z 10,0] [--seed 1] [--device 0]
//             [--tables DIR] [--max-steps N] [--quiet]
// Initial conditions: Zel'dovich on the device (cube_ic_zeldovich).  At each
// redshift of --z the state is written in the reference's checkpoint format
// (cube_checkpoint_write); the run ends after the last one.  One line per
// step goes to stdout.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cube_gpu.h"

namespace {

const float kPi = 4.0f * std::atan(1.0f);  // pi=4*atan(1.) in real(4), parameters.f90:67
const float kGG = (1.0f / 6.0f) / kPi;      // GG=1.0/6.0/pi, variables.f90:15

struct Cosmo {
  float omega_m = 0.3f, omega_l = 0.7f, wde = -1.0f;
};

// expansion (timestep.f90:133-177): a third-order Friedmann step over dt0 in
// two halves; the derivatives in real(8), the increments real(4).  The
// literal 4.0/9.0 is a default-real quotient widened to real(8).
void expansion(const Cosmo& cs, float a0, float dt0, float* da1, float* da2) {
  const float om = cs.omega_m, ol = cs.omega_l, w = cs.wde;
  const float dt_x = dt0 / 2.0f;
  const double omhsq = (double)(4.0f / 9.0f);
  const double e3w = (double)(-3.0f * w);
  const double curv = (double)((1.0f - om) - ol);
  auto half = [&](double ax) -> float {
    const double a3rlm = std::pow(ax, e3w) * (double)ol / (double)om;
    const double arkm = ax * curv / (double)om;
    const double adot = std::sqrt(omhsq * std::pow(ax, 3.0) * (1.0 + arkm + a3rlm));
    const double addot = std::pow(ax, 2.0) * omhsq * (1.5 + 2.0 * arkm + 1.5 * (double)(1.0f - w) * a3rlm);
    const double atdot = ax * adot * omhsq *
                         (3.0 + 6.0 * arkm + 1.5 * (double)(2.0f - 3.0f * w) * (double)(1.0f - w) * a3rlm);
    const double dx = (double)dt_x;
    return (float)(adot * dx + (addot * std::pow(dx, 2.0)) / 2.0 + (atdot * std::pow(dx, 3.0)) / 6.0);
  };
  *da1 = half((double)a0);
  *da2 = half((double)(a0 + *da1));
}

// The scalar module state of variables.f90 / sim that the step loop touches.
struct TimeState {
  Cosmo cs;
  float a = 0.02f, t = 0.f, tau = 0.f, dt = 0.f, dt_old = 0.f, da = 0.f, a_mid = 0.f;
  int64_t istep = 0;
  float dt_fine = 1000.f, dt_coarse = 1000.f, dt_pp = 1000.f, dt_vmax = 1000.f;
  float vz_max = 0.f;
  float ra_max = 0.2f, dt_max = 1.0f;
  std::vector<float> z_checkpoints;
  size_t cur_checkpoint = 0;
  bool checkpoint_step = false, final_step = false;

  // timestep (timestep.f90:1-92) for one image
  void timestep() {
    dt_old = dt;
    istep++;
    float dt_e = dt_max, d1, d2;
    for (int ntry = 1;; ntry++) {
      expansion(cs, a, dt_e, &d1, &d2);
      float dda = d1 + d2;
      float ra = dda / (a + dda);
      if (ra > ra_max)
        dt_e = dt_e * (ra_max / ra);
      else
        break;
      if (ntry > 10) break;
    }
    float d = std::fmin(std::fmin(std::fmin(dt_e, dt_fine), std::fmin(dt_coarse, dt_pp)), std::fmin(dt_vmax, 1000.f));
    expansion(cs, a, d, &d1, &d2);
    float dda = d1 + d2;
    checkpoint_step = false;
    if (cur_checkpoint < z_checkpoints.size()) {
      const float z_next = z_checkpoints[cur_checkpoint];
      const float a_next = 1.0f / (1.0f + z_next);
      if (dda >= a_next - a) {
        checkpoint_step = true;
        if (cur_checkpoint + 1 == z_checkpoints.size()) final_step = true;
        for (int n = 0; std::fabs((a + dda) / a_next - 1.0f) >= 1e-6f && n < 100; n++) {
          d = d * ((a_next - a) / dda);
          expansion(cs, a, d, &d1, &d2);
          dda = d1 + d2;
        }
      }
    }
    a_mid = a + (dda / 2.0f);
    tau = tau + d;
    t = t + d;
    a = a + dda;
    da = dda;
    dt = d;
  }

  // dt constraints from the device maxima (pm.f90:395-398; ext_pp_force.f90:141)
  void constrain(const cube_stats& pm, const cube_stats* pp, int ncell) {
    const float am = a_mid;
    if (pm.f2_max_fine > 0.f) dt_fine = std::sqrt(1.0f / (std::sqrt(pm.f2_max_fine) * am * kGG));
    if (pm.f2_max_coarse > 0.f) dt_coarse = std::sqrt((float)ncell / (std::sqrt(pm.f2_max_coarse) * am * kGG));
    const float vm = std::fmax(std::fmax(pm.vmax[0], pm.vmax[1]), pm.vmax[2]);
    if (vm > 0.f) dt_vmax = (0.9f * 20.0f) / vm;
    vz_max = pm.vmax[2];
    if (pp && pp->f2_max_pp > 0.f) dt_pp = 1.0f * std::sqrt(1.0f) / (std::sqrt(pp->f2_max_pp) * am * kGG);
  }
};

bool read_table(const std::string& path, std::vector<float>& out, size_t n) {
  out.assign(n, 0.f);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  size_t got = std::fread(out.data(), sizeof(float), n, f);
  std::fclose(f);
  return got == n;
}

int die(cube_ctx* c, int rc, const char* what) {
  std::fprintf(stderr, "cube_main: %s failed (status %d): %s\n", what, rc, c ? cube_last_error(c) : "");
  if (c) cube_destroy(c);
  return 1;
}

std::vector<float> parse_list(const char* s) {
  std::vector<float> v;
  std::string str(s);
  size_t i = 0;
  while (i <= str.size()) {
    size_t j = str.find(',', i);
    if (j == std::string::npos) j = str.size();
    if (j > i) v.push_back(std::strtof(str.substr(i, j - i).c_str(), nullptr));
    i = j + 1;
  }
  return v;
}

}  // namespace

int main(int argc, char** argv) {
  int nc = 32, nnt = 1, np_nc = 2, pp = 0, device = 0, quiet = 0;
  float box = 200.f, rsoft = 0.1f, z_init = 49.f;
  unsigned seed = 1;
  long max_steps = 100000;
  std::vector<float> zs = {0.f};
  std::string out, tables;
  for (int i = 1; i < argc; i++) {
    std::string k(argv[i]);
    auto val = [&]() -> const char* {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "cube_main: %s needs a value\n", k.c_str());
        std::exit(2);
      }
      return argv[++i];
    };
    if (k == "--nc") nc = std::atoi(val());
    else if (k == "--nnt") nnt = std::atoi(val());
    else if (k == "--np-nc") np_nc = std::atoi(val());
    else if (k == "--box") box = std::strtof(val(), nullptr);
    else if (k == "--pp") pp = std::atoi(val());
    else if (k == "--rsoft") rsoft = std::strtof(val(), nullptr);
    else if (k == "--z-init") z_init = std::strtof(val(), nullptr);
    else if (k == "--z") zs = parse_list(val());
    else if (k == "--seed") seed = (unsigned)std::strtoul(val(), nullptr, 10);
    else if (k == "--device") device = std::atoi(val());
    else if (k == "--tables") tables = val();
    else if (k == "--out") out = val();
    else if (k == "--max-steps") max_steps = std::atol(val());
    else if (k == "--quiet") quiet = 1;
    else {
      std::fprintf(stderr, "cube_main: unknown option %s\n", k.c_str());
      return 2;
    }
  }
  if (out.empty() || zs.empty() || nc <= 0 || nnt <= 0 || nc % nnt || np_nc <= 0) {
    std::fprintf(stderr, "usage: cube_main --out DIR [--nc N] [--nnt N] [--np-nc N] [--box L] [--pp 0|1] "
                         "[--rsoft R] [--z-init Z] [--z Z1,Z2,...] [--seed S] [--tables DIR] [--max-steps N]\n");
    return 2;
  }
  if (tables.empty()) {  // the package's data directory beside host/
    std::string self(argv[0]);
    size_t s = self.rfind('/');
    std::string dir = s == std::string::npos ? "." : self.substr(0, s);
    tables = dir + "/../data";
  }
  std::vector<float> fine, coarse;
  if (!read_table(tables + "/fine_force_table.f32", fine, 3 * 16 * 16 * 16) ||
      !read_table(tables + "/coarse_force_table.f32", coarse, 3 * 4 * 4 * 4)) {
    std::fprintf(stderr, "cube_main: cannot read the force tables in %s\n", tables.c_str());
    return 1;
  }

  // parameters.f90: ncell 4, ncb 6, int8 positions, int16 velocities; the
  // particle mass makes the mean fine-cell density 1 (initial_conditions.f90:868)
  const int64_t npg = (int64_t)nc * np_nc * (int64_t)nc * np_nc * (int64_t)nc * np_nc;
  cube_params p{};
  p.nc = nc;
  p.nnt = nnt;
  p.ncell = 4;
  p.ncb = 6;
  p.izipx = 1;
  p.izipv = 2;
  p.nf_cutoff = 16;
  p.pp_range = 1;
  p.pp_on = pp;
  p.with_pid = 1;
  p.rsoft = rsoft;
  p.mass_p = (float)std::pow(4.0 / np_nc, 3);
  p.np_max = npg + npg / 4 + 4096;
  cube_ctx* c = nullptr;
  int rc = cube_create(&p, fine.data(), coarse.data(), device, &c);
  if (rc) return die(c, rc, "cube_create");

  cube_cosmology cosmo{};
  cosmo.box = box;
  cosmo.omega_m = 0.3f;
  cosmo.omega_l = 0.7f;
  cosmo.h0 = 0.7f;
  cosmo.s8 = 0.8f;
  cosmo.n_s = 0.96f;
  cosmo.omega_b = 0.045f;
  cosmo.np_nc = np_nc;
  float sigma = 0.f, vm[3] = {0.f, 0.f, 0.f};
  if ((rc = cube_ic_zeldovich(c, &cosmo, z_init, seed, &sigma, vm))) return die(c, rc, "cube_ic_zeldovich");

  TimeState ts;
  ts.cs.omega_m = cosmo.omega_m;
  ts.cs.omega_l = cosmo.omega_l;
  ts.a = 1.0f / (1.0f + z_init);
  ts.z_checkpoints = zs;
  ts.vz_max = vm[2];
  ts.dt_vmax = 18.0f / std::fmax(std::fmax(vm[0], vm[1]), vm[2]);

  cube_sim_header hdr{};
  hdr.npglobal = npg;
  hdr.nn = 1;
  hdr.mass_p_cdm = p.mass_p;
  hdr.box = box;
  hdr.h0 = cosmo.h0;
  hdr.omega_m = cosmo.omega_m;
  hdr.omega_l = cosmo.omega_l;
  hdr.s8 = cosmo.s8;
  hdr.z_i = z_init;
  hdr.z_i_nu = z_init;

  cube_stats su{}, sp{}, sm{};
  for (long step = 0; step < max_steps; step++) {
    ts.timestep();
    if ((rc = cube_update_x(c, ts.dt_old, ts.dt, ts.vz_max, &su))) return die(c, rc, "update_x");
    if ((rc = cube_buffer_grid(c)) || (rc = cube_buffer_x(c))) return die(c, rc, "buffer_grid/buffer_x");
    if (pp) {
      if ((rc = cube_pp_particle_mesh(c, ts.a_mid, ts.dt, &sp, &sm))) return die(c, rc, "ext_pp_force + particle_mesh");
    } else if ((rc = cube_particle_mesh(c, ts.a_mid, ts.dt, &sm))) {
      return die(c, rc, "particle_mesh");
    }
    if ((rc = cube_buffer_v(c))) return die(c, rc, "buffer_v");
    ts.constrain(sm, pp ? &sp : nullptr, p.ncell);
    if (!quiet)
      std::printf("step %ld a %.6f z %.4f dt %.6g nplocal %lld npairs %lld sigma_vi %.6g vmax %.5g %.5g %.5g\n",
                  (long)ts.istep, ts.a, 1.0 / ts.a - 1.0, ts.dt, (long long)su.nplocal, (long long)sp.npairs,
                  su.sigma_vi_new, sm.vmax[0], sm.vmax[1], sm.vmax[2]);
    if (ts.checkpoint_step) {
      // the half drift that brings positions to the checkpoint's time
      // (main.f90:121-123), then the checkpoint
      ts.dt_old = 0.f;
      if ((rc = cube_update_x(c, ts.dt_old, ts.dt, ts.vz_max, &su))) return die(c, rc, "update_x (checkpoint)");
      const float z = ts.z_checkpoints[ts.cur_checkpoint];
      hdr.timestep = ts.istep;
      hdr.cur_checkpoint = (int64_t)ts.cur_checkpoint + 1;
      hdr.a = ts.a;
      hdr.t = ts.t;
      hdr.tau = ts.tau;
      hdr.dt_fine = ts.dt_fine;
      hdr.dt_coarse = ts.dt_coarse;
      hdr.dt_pp = ts.dt_pp;
      hdr.dt_vmax = ts.dt_vmax;
      hdr.vz_max = ts.vz_max;
      hdr.vsim2phys = (1.5f / ts.a) * box * 100.f * std::sqrt(cosmo.omega_m) / (float)(nc * 4);
      if ((rc = cube_checkpoint_write(c, out.c_str(), z, 1, &hdr))) return die(c, rc, "checkpoint");
      if (!quiet) std::printf("checkpoint z %.3f written to %s\n", z, out.c_str());
      ts.cur_checkpoint++;
      if ((rc = cube_buffer_grid(c)) || (rc = cube_buffer_x(c)) || (rc = cube_buffer_v(c)))
        return die(c, rc, "buffers (checkpoint)");
      if (ts.final_step) break;
      ts.dt = 0.f;
    }
  }
  cube_destroy(c);
  return ts.final_step ? 0 : 3;
}
