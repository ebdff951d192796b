// Flat binary training-set files of the source surrogate (host code).
//
// Layout: the 8 bytes "SBZTRN01", int32 nin, int32 nout, int64 nrows, then nrows rows of
// nin + nout little-endian float32 (the inputs, then the targets).  Rows are appended shard by
// shard as the solver produces them (the header's row count is rewritten after each append), and
// read back in any contiguous range, so a training set larger than host memory can be streamed.
// This is the training-data counterpart of the SBZMLP01 weight files (the reference has no
// surrogate; its parameter_updater, src/solve.jl:271-306, is the batched parameter path that
// generates the data).
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include "../../include/symboltz_gb300.h"

namespace sbz {
int capi_fail(int code, const char* msg);
}

namespace {

constexpr char kMagic[8] = {'S', 'B', 'Z', 'T', 'R', 'N', '0', '1'};
constexpr long kHeader = 8 + 4 + 4 + 8;

int fail(const std::string& msg) { return sbz::capi_fail(SBZ_ERR_ARG, msg.c_str()); }

bool read_header(FILE* f, int32_t* nin, int32_t* nout, int64_t* nrows) {
  char magic[8];
  return std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kMagic, 8) == 0 && std::fread(nin, 4, 1, f) == 1 &&
         std::fread(nout, 4, 1, f) == 1 && std::fread(nrows, 8, 1, f) == 1 && *nin > 0 && *nout > 0 && *nrows >= 0;
}

}  // namespace

extern "C" {

int sbz_trainset_append(const char* path, int nin, int nout, long long n, const float* X, const float* Y) {
  if (!path || nin <= 0 || nout <= 0 || n < 0 || (n > 0 && (!X || !Y))) return fail("sbz_trainset_append: bad arguments");
  FILE* f = std::fopen(path, "r+b");
  int32_t fin = nin, fout = nout;
  int64_t rows = 0;
  if (f) {
    if (!read_header(f, &fin, &fout, &rows)) { std::fclose(f); return fail(std::string("not a training-set file: ") + path); }
    if (fin != nin || fout != nout) {
      std::fclose(f);
      return fail("sbz_trainset_append: the file holds rows of " + std::to_string(fin) + " inputs and " + std::to_string(fout) +
                  " targets");
    }
  } else {
    f = std::fopen(path, "w+b");
    if (!f) return fail(std::string("cannot create ") + path);
    if (std::fwrite(kMagic, 1, 8, f) != 8 || std::fwrite(&fin, 4, 1, f) != 1 || std::fwrite(&fout, 4, 1, f) != 1 ||
        std::fwrite(&rows, 8, 1, f) != 1) {
      std::fclose(f);
      return fail(std::string("write failed: ") + path);
    }
  }
  const size_t w = (size_t)nin + nout;
  if (std::fseek(f, kHeader + (long)(rows * (int64_t)w * 4), SEEK_SET) != 0) { std::fclose(f); return fail("seek failed"); }
  std::vector<float> buf;
  const long long chunk = 1 << 16;
  bool ok = true;
  for (long long r0 = 0; r0 < n && ok; r0 += chunk) {
    const long long m = n - r0 < chunk ? n - r0 : chunk;
    buf.resize((size_t)m * w);
    for (long long r = 0; r < m; ++r) {
      std::memcpy(&buf[(size_t)r * w], X + (size_t)(r0 + r) * nin, sizeof(float) * nin);
      std::memcpy(&buf[(size_t)r * w + nin], Y + (size_t)(r0 + r) * nout, sizeof(float) * nout);
    }
    ok = std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
  }
  rows += n;
  ok = ok && std::fseek(f, 16, SEEK_SET) == 0 && std::fwrite(&rows, 8, 1, f) == 1;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SBZ_OK : fail(std::string("write failed: ") + path);
}

int sbz_trainset_info(const char* path, int* nin, int* nout, long long* nrows) {
  if (!path || !nin || !nout || !nrows) return fail("sbz_trainset_info: bad arguments");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(std::string("cannot read ") + path);
  int32_t a, b;
  int64_t r;
  const bool ok = read_header(f, &a, &b, &r);
  std::fclose(f);
  if (!ok) return fail(std::string("not a training-set file: ") + path);
  *nin = a; *nout = b; *nrows = r;
  return SBZ_OK;
}

int sbz_trainset_read(const char* path, long long first, long long n, float* X, float* Y) {
  if (!path || first < 0 || n < 0 || (n > 0 && (!X || !Y))) return fail("sbz_trainset_read: bad arguments");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(std::string("cannot read ") + path);
  int32_t nin, nout;
  int64_t rows;
  if (!read_header(f, &nin, &nout, &rows)) { std::fclose(f); return fail(std::string("not a training-set file: ") + path); }
  if (first + n > rows) {
    std::fclose(f);
    return fail("sbz_trainset_read: rows " + std::to_string(first) + ".." + std::to_string(first + n) + " past the " +
                std::to_string(rows) + " in the file");
  }
  const size_t w = (size_t)nin + nout;
  bool ok = std::fseek(f, kHeader + (long)(first * (int64_t)w * 4), SEEK_SET) == 0;
  std::vector<float> buf;
  const long long chunk = 1 << 16;
  for (long long r0 = 0; r0 < n && ok; r0 += chunk) {
    const long long m = n - r0 < chunk ? n - r0 : chunk;
    buf.resize((size_t)m * w);
    ok = std::fread(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    for (long long r = 0; ok && r < m; ++r) {
      std::memcpy(X + (size_t)(r0 + r) * nin, &buf[(size_t)r * w], sizeof(float) * nin);
      std::memcpy(Y + (size_t)(r0 + r) * nout, &buf[(size_t)r * w + nin], sizeof(float) * nout);
    }
  }
  std::fclose(f);
  return ok ? SBZ_OK : fail(std::string("truncated training-set file: ") + path);
}

}  // extern "C"
