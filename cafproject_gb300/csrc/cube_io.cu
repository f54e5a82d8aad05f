// cube_io.cu -- checkpoints in the reference's file format (checkpoint.f90:
// 10-50, read back by particle_initialization.f90:34-64): one directory per
// image, files <z>_<name>_<image>.bin written with Fortran stream access, i.e.
// raw arrays in their Fortran layouts:
//   info  sim_header (parameters.f90:136-160), 17 int64 + 22 real(4), 224 bytes
//   xp    xp(3,nplocal)  int8/int16        vp  vp(3,nplocal) int8/int16
//   np    rhoc(nt,nt,nt,nnt,nnt,nnt) int32  vc  vfield(3,nt,...,nnt) real(4)
//   id    pid(nplocal) int32 (written when the context carries particle ids)
// A context linked to another (the second species) writes and reads the
// *_nu files; its counts, formats and sigma_vi live in the owner's header.
// <z> is z formatted as Fortran f7.3 with the blanks removed (z2str,
// basic_functions.fh:36-42).  The state moves through pinned host buffers and
// the files are written (read) by one host thread each, as the reference's
// OpenMP sections do.
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "cube_internal.cuh"

static_assert(sizeof(cube_sim_header) == 224, "sim_header is 17 int64 + 22 real(4) without padding");

namespace {

std::string f73(float z) {
  char b[64];
  std::snprintf(b, sizeof b, "%7.3f", (double)z);
  std::string s(b);
  if (s.size() > 7) s = "*******";  // Fortran prints asterisks when f7.3 overflows
  size_t i = s.find_first_not_of(' ');
  return i == std::string::npos ? s : s.substr(i);
}

std::string file_name(const char* dir, float z, int image, const char* what, bool nu = false) {
  std::string d(dir);
  if (!d.empty() && d.back() != '/') d += '/';
  return d + f73(z) + "_" + what + (nu ? "_nu" : "") + "_" + std::to_string(image) + ".bin";
}

struct FileJob {
  std::string path;
  void* data;
  size_t bytes;
  bool ok = false;
};

void run_jobs(std::vector<FileJob>& jobs, bool write) {
  std::vector<std::thread> th;
  for (FileJob& j : jobs) {
    th.emplace_back([&j, write] {
      FILE* f = std::fopen(j.path.c_str(), write ? "wb" : "rb");
      if (!f) return;
      size_t n = write ? std::fwrite(j.data, 1, j.bytes, f) : std::fread(j.data, 1, j.bytes, f);
      if (!write) {  // the file must hold exactly the expected bytes
        unsigned char extra;
        if (std::fread(&extra, 1, 1, f) != 0) n = (size_t)-1;
      }
      j.ok = std::fclose(f) == 0 && n == j.bytes;
    });
  }
  for (std::thread& t : th) t.join();
}

struct Pinned {
  void* p = nullptr;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

}  // namespace

extern "C" int cube_checkpoint_write(cube_ctx* c, const char* dir, float z, int image, const cube_sim_header* hdr) {
  if (!c || !dir || !hdr || image < 1) return CUBE_ERR_ARG;
  if (!c->have_state) return cube_fail(c, CUBE_ERR_STATE, "no state uploaded");
  CUBE_CUDA(c, cudaSetDevice(c->device));
  const int64_t np = c->np, ncell = c->ncells;
  const size_t bx = 3 * (size_t)np * c->p.izipx, bv = 3 * (size_t)np * c->p.izipv, bi = 4 * (size_t)np;
  const size_t br = 4 * (size_t)ncell, bf = 12 * (size_t)ncell;
  Pinned h;
  CUBE_CUDA(c, cudaMallocHost(&h.p, bx + bv + bi + br + bf + 64));
  unsigned char* base = static_cast<unsigned char*>(h.p);
  unsigned char *hx = base, *hv = hx + bx, *hi = hv + bv, *hr = hi + bi, *hf = hr + br;
  int64_t n_out = 0;
  int r = cube_state_out(c, &n_out, hx, hv, c->p.with_pid ? (int32_t*)hi : nullptr, (int32_t*)hr, (float*)hf);
  if (r) return r;
  cube_sim_header s = *hdr;
  s.nplocal = np;
  s.izipx = c->p.izipx;
  s.izipv = c->p.izipv;
  s.nnt = c->p.nnt;
  s.nt = c->nt;
  s.ncell = c->p.ncell;
  s.ncb = c->p.ncb;
  s.image = image;
  s.sigma_vi = c->sigma_vi;  // checkpoint.f90:31
  // the second species' fields of the header come from its live state, as
  // the reference writes sigma_vi_nu (CUBEnu checkpoint.f90:32), so the info
  // file always matches the *_nu files written beside it
  if (c->linked && c->linked->have_state) {
    const cube_ctx* nu = c->linked;
    s.nplocal_nu = nu->np;
    s.izipx_nu = nu->p.izipx;
    s.izipv_nu = nu->p.izipv;
    s.sigma_vi_nu = nu->sigma_vi;
  }
  // the linked species writes xp_nu, vp_nu, np_nu, vc_nu, id_nu (checkpoint.f90:19-23, 55-70);
  // its counts travel in the owner's header (nplocal_nu)
  const bool nu = c->owner != nullptr;
  std::vector<FileJob> jobs = {{file_name(dir, z, image, "xp", nu), hx, bx},
                               {file_name(dir, z, image, "vp", nu), hv, bv},
                               {file_name(dir, z, image, "np", nu), hr, br},
                               {file_name(dir, z, image, "vc", nu), hf, bf}};
  if (!nu) jobs.insert(jobs.begin(), FileJob{file_name(dir, z, image, "info"), &s, sizeof s});
  if (c->p.with_pid) jobs.push_back({file_name(dir, z, image, "id", nu), hi, bi});
  run_jobs(jobs, true);
  for (const FileJob& j : jobs)
    if (!j.ok) return cube_fail(c, CUBE_ERR_ARG, "could not write " + j.path);
  return CUBE_OK;
}

extern "C" int cube_checkpoint_read(cube_ctx* c, const char* dir, float z, int image, cube_sim_header* hdr) {
  if (!c || !dir || image < 1) return CUBE_ERR_ARG;
  CUBE_CUDA(c, cudaSetDevice(c->device));
  cube_sim_header s;
  std::vector<FileJob> head = {{file_name(dir, z, image, "info"), &s, sizeof s}};
  run_jobs(head, false);
  if (!head[0].ok) return cube_fail(c, CUBE_ERR_ARG, "could not read " + head[0].path);
  // the linked species reads the *_nu files with its counts, formats and
  // sigma from the owner's header (particle_initialization.f90:35-45, 65-77)
  const bool nu = c->owner != nullptr;
  const int64_t hz = nu ? s.izipx_nu : s.izipx, hv_ = nu ? s.izipv_nu : s.izipv, hn = nu ? s.nplocal_nu : s.nplocal;
  if (hz != c->p.izipx || hv_ != c->p.izipv) return cube_fail(c, CUBE_ERR_ARG, "zip format incompatible");
  if (s.nt != c->nt || s.nnt != c->p.nnt) return cube_fail(c, CUBE_ERR_ARG, "tile geometry differs from the context");
  if (hn < 0 || hn > c->p.np_max) return cube_fail(c, CUBE_ERR_IMAGE_OVERFLOW, "nplocal exceeds np_max");
  const int64_t np = hn, ncell = c->ncells;
  const size_t bx = 3 * (size_t)np * c->p.izipx, bv = 3 * (size_t)np * c->p.izipv, bi = 4 * (size_t)np;
  const size_t br = 4 * (size_t)ncell, bf = 12 * (size_t)ncell;
  Pinned h;
  CUBE_CUDA(c, cudaMallocHost(&h.p, bx + bv + bi + br + bf + 64));
  unsigned char* base = static_cast<unsigned char*>(h.p);
  unsigned char *hx = base, *hv = hx + bx, *hi = hv + bv, *hr = hi + bi, *hf = hr + br;
  std::vector<FileJob> jobs = {{file_name(dir, z, image, "xp", nu), hx, bx},
                               {file_name(dir, z, image, "vp", nu), hv, bv},
                               {file_name(dir, z, image, "np", nu), hr, br},
                               {file_name(dir, z, image, "vc", nu), hf, bf}};
  if (c->p.with_pid) jobs.push_back({file_name(dir, z, image, "id", nu), hi, bi});
  run_jobs(jobs, false);
  for (const FileJob& j : jobs)
    if (!j.ok) return cube_fail(c, CUBE_ERR_ARG, "could not read " + j.path + " (missing or wrong size)");
  int r = cube_state_in(c, np, hx, hv, c->p.with_pid ? (const int32_t*)hi : nullptr, (const int32_t*)hr,
                        (const float*)hf);
  if (r) return r;
  c->sigma_vi = nu ? s.sigma_vi_nu : s.sigma_vi;  // particle_initialization.f90:38-39
  if (hdr) *hdr = s;
  return CUBE_OK;
}
