// save_npz / load_npz of scirs2-sparse (src/io.rs:49-269) for CSR arrays:
// the reference's own little-endian record, not SciPy's zip archive:
//   u64 len, len bytes     format marker ("csr_array")
//   u64 rows, u64 cols     shape
//   u64 len, len values    data (the value type's bytes)
//   u64 len, len u64       indices
//   u64 len, len u64       indptr
// Loading validates like CsrArray::new and uploads straight into a device
// CSR (sx_csr_from_raw).  Errors follow the reference: I/O failures are
// ComputationError("IO error: ...") with Rust's io::Error text, an unknown
// marker is ConversionError("Unknown format: ...").
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "sx_internal.h"

namespace sx {
namespace {

int io_error(const std::string& what) { return set_error(SX_ERR_COMPUTATION, "Computation error: IO error: " + what); }
// std::io::Error's Display for an OS error
std::string os_error(int e) { return std::string(std::strerror(e)) + " (os error " + std::to_string(e) + ")"; }
const char* kEof = "failed to fill whole buffer";  // read_exact at end of file

struct Reader {
  FILE* f = nullptr;
  uint64_t left = 0;  // bytes not yet read
  int read(void* dst, uint64_t n) {
    if (n > left) return io_error(kEof);
    if (n > 0 && std::fread(dst, 1, (size_t)n, f) != (size_t)n) return io_error(kEof);
    left -= n;
    return SX_OK;
  }
  int u64(uint64_t* v) {
    unsigned char b[8];
    SX_CHECK(read(b, 8));
    uint64_t x = 0;
    for (int i = 7; i >= 0; --i) x = (x << 8) | b[i];
    *v = x;
    return SX_OK;
  }
  // read_array: u64 length, then length * elem bytes (a length beyond the
  // file ends the read as read_exact does)
  int array(std::vector<unsigned char>& out, uint64_t* len, size_t elem) {
    SX_CHECK(u64(len));
    if (*len > left / elem) return io_error(kEof);
    out.resize((size_t)(*len * elem));
    return read(out.data(), *len * elem);
  }
};

// String::from_utf8's check, with Utf8Error's Display on failure
bool utf8_error(const std::vector<unsigned char>& s, std::string* msg) {
  const size_t n = s.size();
  size_t i = 0;
  auto cont = [&](size_t k) { return k < n && (s[k] & 0xC0) == 0x80; };
  while (i < n) {
    const unsigned char c = s[i];
    if (c < 0x80) {
      ++i;
      continue;
    }
    int w = 0;
    if (c >= 0xC2 && c <= 0xDF) w = 2;
    else if (c >= 0xE0 && c <= 0xEF) w = 3;
    else if (c >= 0xF0 && c <= 0xF4) w = 4;
    auto fail = [&](int len) {
      *msg = len == 0 ? "incomplete utf-8 byte sequence from index " + std::to_string(i)
                      : "invalid utf-8 sequence of " + std::to_string(len) + " bytes from index " + std::to_string(i);
      return true;
    };
    if (w == 0) return fail(1);
    if (i + 1 >= n) return fail(0);
    const unsigned char c1 = s[i + 1];
    bool ok1;
    if (w == 2) ok1 = (c1 & 0xC0) == 0x80;
    else if (c == 0xE0) ok1 = c1 >= 0xA0 && c1 <= 0xBF;
    else if (c == 0xED) ok1 = c1 >= 0x80 && c1 <= 0x9F;
    else if (w == 3) ok1 = c1 >= 0x80 && c1 <= 0xBF;
    else if (c == 0xF0) ok1 = c1 >= 0x90 && c1 <= 0xBF;
    else if (c == 0xF4) ok1 = c1 >= 0x80 && c1 <= 0x8F;
    else ok1 = c1 >= 0x80 && c1 <= 0xBF;
    if (!ok1) return fail(1);
    if (w == 2) {
      i += 2;
      continue;
    }
    if (i + 2 >= n) return fail(0);
    if (!cont(i + 2)) return fail(2);
    if (w == 3) {
      i += 3;
      continue;
    }
    if (i + 3 >= n) return fail(0);
    if (!cont(i + 3)) return fail(3);
    i += 4;
  }
  return false;
}

void put_u64(std::vector<unsigned char>& b, uint64_t v) {
  for (int i = 0; i < 8; ++i) b.push_back((unsigned char)(v >> (8 * i)));
}

}  // namespace
}  // namespace sx

using namespace sx;

extern "C" {

int sx_csr_save_npz(sx_ctx ctx, sx_op a, const char* path) {
  if (!ctx || !a || !path) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (a->kind != SX_OP_CSR) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: not a CSR operator");
  const int64_t n = a->nrows, nnz = a->csr.nnz;
  const size_t w = elt_size(a->dtype);
  std::vector<uint64_t> ip((size_t)n + 1), ix((size_t)std::max<int64_t>(nnz, 1));
  std::vector<unsigned char> data((size_t)std::max<int64_t>(nnz, 1) * w);
  SX_CHECK(sx_csr_download(ctx, a, ip.data(), ix.data(), data.data()));
  FILE* f = std::fopen(path, "wb");
  if (!f) return io_error(os_error(errno));
  std::vector<unsigned char> head;
  const char* marker = "csr_array";  // io.rs:22
  put_u64(head, std::strlen(marker));
  head.insert(head.end(), marker, marker + std::strlen(marker));
  put_u64(head, (uint64_t)n);
  put_u64(head, (uint64_t)a->ncols);
  put_u64(head, (uint64_t)nnz);
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  // values in the value type's little-endian bytes (the reference writes the
  // machine's bytes; every supported host is little-endian)
  if (ok && nnz > 0) ok = std::fwrite(data.data(), 1, (size_t)nnz * w, f) == (size_t)nnz * w;
  std::vector<unsigned char> tail;
  put_u64(tail, (uint64_t)nnz);
  for (int64_t k = 0; k < nnz; ++k) put_u64(tail, ix[k]);
  put_u64(tail, (uint64_t)n + 1);
  for (int64_t k = 0; k <= n; ++k) put_u64(tail, ip[k]);
  if (ok) ok = std::fwrite(tail.data(), 1, tail.size(), f) == tail.size();
  const int e = errno;
  if (std::fclose(f) != 0) ok = false;
  if (!ok) return io_error(os_error(e ? e : EIO));
  return clear_error();
}

int sx_csr_load_npz(sx_ctx ctx, sx_dtype dtype, const char* path, sx_op* out) {
  if (!ctx || !path || !out) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: null");
  if (dtype != SX_F32 && dtype != SX_F64) return set_error(SX_ERR_INVALID_ARGUMENT, "Invalid argument: dtype");
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return io_error(os_error(errno));
  Reader r;
  r.f = f;
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  r.left = size > 0 ? (uint64_t)size : 0;
  int rc = SX_OK;
  std::vector<unsigned char> fmt, data, idx, ptr;
  uint64_t flen = 0, rows = 0, cols = 0, dlen = 0, ilen = 0, plen = 0;
  std::string format;
  do {
    // io.rs:220-233: marker, shape, data, indices (in that order)
    if ((rc = r.u64(&flen))) break;
    if (flen > r.left) {
      rc = io_error(kEof);
      break;
    }
    fmt.resize((size_t)flen);
    if ((rc = r.read(fmt.data(), flen))) break;
    std::string umsg;
    if (utf8_error(fmt, &umsg)) {
      rc = io_error(umsg);
      break;
    }
    format.assign(fmt.begin(), fmt.end());
    if ((rc = r.u64(&rows))) break;
    if ((rc = r.u64(&cols))) break;
    if ((rc = r.array(data, &dlen, elt_size(dtype)))) break;
    if ((rc = r.array(idx, &ilen, 8))) break;
    if (format == "csr_array") {
      if ((rc = r.array(ptr, &plen, 8))) break;
    } else if (format == "csc_array" || format == "coo_array" || format == "dok_array") {
      rc = set_error(SX_ERR_NOT_IMPLEMENTED,
                     "Feature not implemented: " + format + " records load only as CSR on the device");
      break;
    } else {
      rc = set_error(SX_ERR_CONVERSION, "Conversion error: Unknown format: " + format);
      break;
    }
  } while (0);
  std::fclose(f);
  if (rc != SX_OK) return rc;
  // CsrArray::new (csr_array.rs:84-88): equal data and indices lengths first
  if (dlen != ilen)
    return set_error(SX_ERR_INCONSISTENT_DATA, "Inconsistent data: data and indices must have the same length");
  std::vector<uint64_t> ipv((size_t)plen), ixv((size_t)ilen);
  for (uint64_t k = 0; k < plen; ++k) {
    uint64_t v = 0;
    for (int b = 7; b >= 0; --b) v = (v << 8) | ptr[(size_t)(k * 8 + b)];
    ipv[k] = v;
  }
  for (uint64_t k = 0; k < ilen; ++k) {
    uint64_t v = 0;
    for (int b = 7; b >= 0; --b) v = (v << 8) | idx[(size_t)(k * 8 + b)];
    ixv[k] = v;
  }
  return sx_csr_from_raw(ctx, dtype, SX_API_CSR_ARRAY, ipv.data(), plen, ixv.data(), data.data(), dlen, rows, cols,
                         out);
}

}  // extern "C"
