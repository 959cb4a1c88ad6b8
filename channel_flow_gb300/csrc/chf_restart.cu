// chf_restart.cu -- restart files in the reference's layout (host code).
//
// The reference writes one Fortran unformatted sequential file per MPI rank
// (output, poiseuilleflow.f90:2460-2504) and reads it back in initial
// (poiseuilleflow.f90:1873-1917):
//   record 1: clamb1n, clamb1nm1, clamb3n, clamb3nm1, au0, w0   each (2, 0:nz) real*8
//   record 2: vnp1, omegaynp1, rhsvn, rhsomegayn, unp1, wnp1    each (0:nx, 0:ny, 0:nz) real*8
// Each record is framed by 4-byte little-endian byte counts (the
// gfortran / ifort default for records below 2 GiB).  Rank id holds the
// streamwise slab of nx + 1 = nnx / nproc interleaved (re, im) slots starting
// at id (nx + 1) (the wavenumbers iapha, poiseuilleflow.f90:132-134), the full
// spanwise and wall-normal extent.  File names follow format 2111
// ('data', i8.8, '_instant.', i3.3, '.dat') with the tag iii = 2 of the
// reference, or format 22211 (adds '_', i8.8 step) when a step is given.
//
// The file is written where the reference calls output: after getnonlinear,
// before the solve, so unp1 / wnp1 hold the previous nonlinear terms.  A run
// restarted from it begins with the solve (the istep = istepbegin iteration,
// poiseuilleflow.f90:222-226).  omega_x / omega_z are not in the file; the
// solve recomputes them.  Only rank 0's mean record is used by the
// reference; every rank's file carries the same values here.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "chf_internal.h"

using namespace chf;

struct chf_handle : public Handle {};

namespace {

// record 2 order of the reference, as field slots of the handle
const int kRec2[6] = {F_V, F_OY, F_RV, F_RG, F_U, F_W};
const int kRec1[6] = {M_CL1N, M_CL1NM1, M_CL3N, M_CL3NM1, M_AU0, M_W0};

std::string restart_name(const char* dir, int tag, int rank, int istep) {
  char buf[96];
  if (istep >= 0)
    std::snprintf(buf, sizeof buf, "data%08d_instant.%03d_%08d.dat", tag, rank, istep);
  else
    std::snprintf(buf, sizeof buf, "data%08d_instant.%03d.dat", tag, rank);
  std::string d = dir && *dir ? dir : ".";
  if (d.back() != '/') d += '/';
  return d + buf;
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

bool put_marker(FILE* f, uint64_t bytes) {
  const uint32_t m = (uint32_t)bytes;  // little-endian host (x86-64, aarch64)
  return std::fwrite(&m, 4, 1, f) == 1;
}

bool get_marker(FILE* f, uint32_t* m) { return std::fread(m, 4, 1, f) == 1; }

int check_layout(Handle* h, int nproc, int tag, int istep) {
  const Dims& d = h->d;
  if (nproc < 1 || nproc > 999 || tag < 0 || tag > 99999999 || istep > 99999999) {
    h->err = "restart: nproc must be 1..999, tag 0..99999999, istep < 1e8";
    return CHF_E_INVALID;
  }
  // the reference's own constraints for nproc ranks (paraandcons.f90:5-8):
  // whole (re, im) pairs per rank and nny / 2 divisible by nproc
  if (d.nnx % (2 * nproc) != 0 || (d.nny / 2) % nproc != 0) {
    h->err = "restart: nnx must be a multiple of 2 nproc and nny / 2 a multiple of nproc";
    return CHF_E_INVALID;
  }
  const uint64_t rec2 = 6ull * (uint64_t)(d.nnx / nproc) * d.nny * d.NZ * sizeof(double);
  if (rec2 > 0x7FFFFFF0ull) {
    h->err = "restart: a record above 2 GiB needs more ranks (subrecords are not written)";
    return CHF_E_INVALID;
  }
  return CHF_OK;
}

}  // namespace

extern "C" int chf_write_restart(chf_handle* h, const char* dir, int nproc, int tag, int istep) {
  if (!h) return CHF_E_INVALID;
  if (!h->uploaded) {
    h->err = "chf_write_restart before chf_upload_state";
    return CHF_E_STATE;
  }
  int rc = check_layout(h, nproc, tag, istep);
  if (rc != CHF_OK) return rc;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  const Dims& d = h->d;
  const size_t fe = 2 * d.field_elems();  // doubles per field
  std::vector<double> mean(6 * 2 * (size_t)d.NZ), fld(6 * fe);
  for (int i = 0; i < 6; ++i) {
    if (!cuda_ok(h, cudaMemcpyAsync(mean.data() + (size_t)i * 2 * d.NZ, h->mean[kRec1[i]],
                                    sizeof(double) * 2 * d.NZ, cudaMemcpyDeviceToHost, h->stream),
                 "restart download") ||
        !cuda_ok(h, cudaMemcpyAsync(fld.data() + (size_t)i * fe, h->f[kRec2[i]], sizeof(double) * fe,
                                    cudaMemcpyDeviceToHost, h->stream),
                 "restart download"))
      return CHF_E_CUDA;
  }
  if (!cuda_ok(h, cudaStreamSynchronize(h->stream), "restart sync")) return CHF_E_CUDA;
  const int w = d.nnx / nproc;  // doubles per (ky, n) row of one rank
  const uint64_t rec1 = mean.size() * sizeof(double);
  const uint64_t rec2 = 6ull * (uint64_t)w * d.nny * d.NZ * sizeof(double);
  for (int r = 0; r < nproc; ++r) {
    const std::string name = restart_name(dir, tag, r, istep);
    File out;
    out.f = std::fopen(name.c_str(), "wb");
    if (!out.f) {
      h->err = "restart: cannot create " + name;
      return CHF_E_INVALID;
    }
    bool ok = put_marker(out.f, rec1) && std::fwrite(mean.data(), 1, rec1, out.f) == rec1 &&
              put_marker(out.f, rec1) && put_marker(out.f, rec2);
    for (int i = 0; ok && i < 6; ++i)
      for (int n = 0; ok && n < d.NZ; ++n)
        for (int ky = 0; ok && ky < d.nny; ++ky) {
          const double* row = fld.data() + (size_t)i * fe + ((size_t)n * d.nny + ky) * d.nnx + (size_t)r * w;
          ok = std::fwrite(row, sizeof(double), w, out.f) == (size_t)w;
        }
    ok = ok && put_marker(out.f, rec2);
    if (!ok || std::fflush(out.f) != 0) {
      h->err = "restart: write failed on " + name;
      return CHF_E_INVALID;
    }
  }
  return CHF_OK;
}

extern "C" int chf_read_restart(chf_handle* h, const char* dir, int nproc, int tag, int istep) {
  if (!h) return CHF_E_INVALID;
  int rc = check_layout(h, nproc, tag, istep);
  if (rc != CHF_OK) return rc;
  if (!cuda_ok(h, cudaSetDevice(h->device), "cudaSetDevice")) return CHF_E_CUDA;
  const Dims& d = h->d;
  const size_t fe = 2 * d.field_elems();
  std::vector<double> mean(6 * 2 * (size_t)d.NZ), fld(6 * fe);
  const int w = d.nnx / nproc;
  const uint64_t rec1 = mean.size() * sizeof(double);
  const uint64_t rec2 = 6ull * (uint64_t)w * d.nny * d.NZ * sizeof(double);
  for (int r = 0; r < nproc; ++r) {
    const std::string name = restart_name(dir, tag, r, istep);
    File in;
    in.f = std::fopen(name.c_str(), "rb");
    if (!in.f) {
      h->err = "restart: cannot open " + name;
      return CHF_E_INVALID;
    }
    uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    std::vector<double> mr(mean.size());
    bool ok = get_marker(in.f, &m0) && m0 == rec1 && std::fread(mr.data(), 1, rec1, in.f) == rec1 &&
              get_marker(in.f, &m1) && m1 == rec1 && get_marker(in.f, &m2) && m2 == rec2;
    for (int i = 0; ok && i < 6; ++i)
      for (int n = 0; ok && n < d.NZ; ++n)
        for (int ky = 0; ok && ky < d.nny; ++ky) {
          double* row = fld.data() + (size_t)i * fe + ((size_t)n * d.nny + ky) * d.nnx + (size_t)r * w;
          ok = std::fread(row, sizeof(double), w, in.f) == (size_t)w;
        }
    ok = ok && get_marker(in.f, &m3) && m3 == rec2;
    if (!ok) {
      h->err = "restart: " + name + " is not a record pair of the expected sizes (grid or nproc differ?)";
      return CHF_E_INVALID;
    }
    if (r == 0) mean = mr;  // the reference uses rank 0's mean arrays
  }
  for (int i = 0; i < 6; ++i) {
    if (!cuda_ok(h, cudaMemcpyAsync(h->mean[kRec1[i]], mean.data() + (size_t)i * 2 * d.NZ,
                                    sizeof(double) * 2 * d.NZ, cudaMemcpyHostToDevice, h->stream),
                 "restart upload") ||
        !cuda_ok(h, cudaMemcpyAsync(h->f[kRec2[i]], fld.data() + (size_t)i * fe, sizeof(double) * fe,
                                    cudaMemcpyHostToDevice, h->stream),
                 "restart upload"))
      return CHF_E_CUDA;
  }
  // omega_x / omega_z are not in the file; the solve recomputes them
  if (!cuda_ok(h, cudaMemsetAsync(h->f[F_OX], 0, sizeof(double) * fe, h->stream), "restart clear") ||
      !cuda_ok(h, cudaMemsetAsync(h->f[F_OZ], 0, sizeof(double) * fe, h->stream), "restart clear") ||
      !cuda_ok(h, cudaStreamSynchronize(h->stream), "restart sync"))
    return CHF_E_CUDA;
  h->uploaded = true;
  return CHF_OK;
}
