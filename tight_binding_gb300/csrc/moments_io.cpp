// moments_io.cpp — binary moment files (header + row-major doubles).
//
// The reference dumps moments and spectra as text columns through
// utils::output_to_file (TB/utils.h:42-69) and writes generate_V_moments'
// upper-triangular V_nm as space-separated text (TB/snippets.h:504-517), six
// significant digits each.  These files keep every bit and the parameters
// needed to reuse them.
#include <cstdio>
#include <cstring>
#include <vector>

#include "tbk_internal.h"

static_assert(sizeof(tbk_moments_header) == 256, "moment file header must stay 256 bytes");

namespace {

const char kMagic[8] = {'T', 'B', 'K', 'M', 'O', 'M', 0, 1};

// FNV-1a, 64-bit (Fowler, Noll, Vo): offset basis 14695981039346656037,
// prime 1099511628211
uint64_t fnv1a(const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  uint64_t h = 14695981039346656037ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ull;
  }
  return h;
}

int64_t n_values(const tbk_moments_header& h) {
  return (int64_t)h.rows * h.cols * (h.is_complex ? 2 : 1);
}

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

int read_header(FILE* f, const char* path, tbk_moments_header* h) {
  if (std::fread(h, sizeof(*h), 1, f) != 1) return tbk::fail(TBK_ERR_INVALID, "%s: short moment file header", path);
  if (std::memcmp(h->magic, kMagic, sizeof(kMagic)) != 0)
    return tbk::fail(TBK_ERR_INVALID, "%s: not a moment file (bad magic)", path);
  if (h->version != 1) return tbk::fail(TBK_ERR_UNSUPPORTED, "%s: moment file version %d", path, h->version);
  if (h->rows < 0 || h->cols < 0) return tbk::fail(TBK_ERR_INVALID, "%s: negative dimensions", path);
  return TBK_OK;
}

}  // namespace

extern "C" {

int tbk_moments_save(const char* path, const tbk_moments_header* header, const double* data) {
  if (!path || !header || (!data && n_values(*header) > 0)) return tbk::fail(TBK_ERR_INVALID, "tbk_moments_save: null argument");
  if (header->rows < 0 || header->cols < 0) return tbk::fail(TBK_ERR_INVALID, "tbk_moments_save: negative dimensions");
  tbk_moments_header h = *header;
  std::memcpy(h.magic, kMagic, sizeof(kMagic));
  h.version = 1;
  h.label[sizeof(h.label) - 1] = 0;
  const size_t bytes = sizeof(double) * (size_t)n_values(h);
  h.checksum = fnv1a(data, bytes);
  File f(path, "wb");
  if (!f.f) return tbk::fail(TBK_ERR_INVALID, "Fail to open %s", path);
  if (std::fwrite(&h, sizeof(h), 1, f.f) != 1 || (bytes && std::fwrite(data, 1, bytes, f.f) != bytes))
    return tbk::fail(TBK_ERR_INVALID, "%s: write failed", path);
  return TBK_OK;
}

int tbk_moments_load_header(const char* path, tbk_moments_header* header) {
  if (!path || !header) return tbk::fail(TBK_ERR_INVALID, "tbk_moments_load_header: null argument");
  File f(path, "rb");
  if (!f.f) return tbk::fail(TBK_ERR_INVALID, "Fail to open %s", path);
  return read_header(f.f, path, header);
}

int tbk_moments_load(const char* path, tbk_moments_header* header, double* data, int64_t capacity) {
  if (!path || !header) return tbk::fail(TBK_ERR_INVALID, "tbk_moments_load: null argument");
  File f(path, "rb");
  if (!f.f) return tbk::fail(TBK_ERR_INVALID, "Fail to open %s", path);
  TBK_TRY(read_header(f.f, path, header));
  const int64_t n = n_values(*header);
  if (n > capacity || (n > 0 && !data))
    return tbk::fail(TBK_ERR_INVALID, "%s: %lld values do not fit the buffer (%lld)", path, (long long)n, (long long)capacity);
  const size_t bytes = sizeof(double) * (size_t)n;
  if (bytes && std::fread(data, 1, bytes, f.f) != bytes) return tbk::fail(TBK_ERR_INVALID, "%s: short moment file", path);
  if (fnv1a(data, bytes) != header->checksum) return tbk::fail(TBK_ERR_INVALID, "%s: checksum mismatch", path);
  return TBK_OK;
}

}  // extern "C"
