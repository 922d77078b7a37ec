// `.wav` files: eigenvalues, 2J labels and Ritz vectors of one problem, the
// format of writeRitzvecs / read_wav / read_appwav
// (src/ShellModel/shellmodel_main.jl:967-1003,1215-1229):
//   int32 neig, int32 Mtot (doubled), float64 E[neig], int32 2J[neig],
//   float64 V[neig][mdim]      (native little-endian, no padding)
// Host code: these calls need no GPU.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/smgpu.h"

namespace {
thread_local std::string g_wav_error;

int wav_fail(int code, const std::string& msg) {
  g_wav_error = msg;
  return code;
}

struct File {
  FILE* f = nullptr;
  explicit File(FILE* x) : f(x) {}
  ~File() {
    if (f) std::fclose(f);
  }
};
}  // namespace

extern "C" {

const char* smgpu_wav_last_error(void) { return g_wav_error.c_str(); }

int smgpu_write_wav(const char* path, long long mdim, int mtot2, int nev, const double* evals, const int* twoJ,
                    const double* vecs) {
  if (!path || mdim < 1 || nev < 1 || !evals || !twoJ || !vecs) return wav_fail(SMGPU_ERR_ARG, "bad arguments");
  File out(std::fopen(path, "wb"));
  if (!out.f) return wav_fail(SMGPU_ERR_IO, std::string("cannot write ") + path);
  const int32_t h[2] = {(int32_t)nev, (int32_t)mtot2};
  std::vector<int32_t> j(twoJ, twoJ + nev);
  bool ok = std::fwrite(h, sizeof(int32_t), 2, out.f) == 2;
  ok = ok && std::fwrite(evals, sizeof(double), (size_t)nev, out.f) == (size_t)nev;
  ok = ok && std::fwrite(j.data(), sizeof(int32_t), (size_t)nev, out.f) == (size_t)nev;
  ok = ok && std::fwrite(vecs, sizeof(double), (size_t)nev * (size_t)mdim, out.f) == (size_t)nev * (size_t)mdim;
  if (!ok) return wav_fail(SMGPU_ERR_IO, std::string("short write to ") + path);
  return SMGPU_OK;
}

int smgpu_read_wav_header(const char* path, long long mdim, int* nev, int* mtot2) {
  if (!path || mdim < 1) return wav_fail(SMGPU_ERR_ARG, "bad arguments");
  File in(std::fopen(path, "rb"));
  if (!in.f) return wav_fail(SMGPU_ERR_IO, std::string("cannot read ") + path);
  int32_t h[2];
  if (std::fread(h, sizeof(int32_t), 2, in.f) != 2 || h[0] < 1)
    return wav_fail(SMGPU_ERR_PARSE, std::string("bad .wav header in ") + path);
  std::fseek(in.f, 0, SEEK_END);
  const long long size = std::ftell(in.f);
  const long long want = 8 + 12ll * h[0] + 8ll * h[0] * mdim;
  if (size != want)
    return wav_fail(SMGPU_ERR_PARSE, std::string(path) + ": size does not match " + std::to_string(h[0]) +
                                         " vectors of dimension " + std::to_string(mdim));
  if (nev) *nev = h[0];
  if (mtot2) *mtot2 = h[1];
  return SMGPU_OK;
}

int smgpu_read_wav(const char* path, long long mdim, int nev_max, double* evals, int* twoJ, double* vecs) {
  int nev = 0, mtot2 = 0;
  int rc = smgpu_read_wav_header(path, mdim, &nev, &mtot2);
  if (rc != SMGPU_OK) return rc;
  if (nev_max < 1) return wav_fail(SMGPU_ERR_ARG, "nev_max must be positive");
  File in(std::fopen(path, "rb"));
  if (!in.f) return wav_fail(SMGPU_ERR_IO, std::string("cannot read ") + path);
  std::fseek(in.f, 8, SEEK_SET);
  std::vector<double> e(nev);
  std::vector<int32_t> j(nev);
  bool ok = std::fread(e.data(), sizeof(double), (size_t)nev, in.f) == (size_t)nev;
  ok = ok && std::fread(j.data(), sizeof(int32_t), (size_t)nev, in.f) == (size_t)nev;
  const int n = nev < nev_max ? nev : nev_max;
  if (ok && vecs) ok = std::fread(vecs, sizeof(double), (size_t)n * (size_t)mdim, in.f) == (size_t)n * (size_t)mdim;
  if (!ok) return wav_fail(SMGPU_ERR_PARSE, std::string("short read from ") + path);
  for (int k = 0; k < n; ++k) {
    if (evals) evals[k] = e[k];
    if (twoJ) twoJ[k] = j[k];
  }
  return SMGPU_OK;
}

}  // extern "C"
