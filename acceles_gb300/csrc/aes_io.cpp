// aes_io.cpp -- host-side data formats on either side of the path: Matrix Market files and the
// ReSparse per-row pruning pass that feeds the packer.
//
// Matrix Market (reference: readMtx/readTuples/undirect/customSort, src/common/utils/utils.hpp
// :331-492 over mmio.hpp; writer write_coo_to_mtx, quantify_util.py:469-477).  The reader maps
// the whole file, splits it at line boundaries and parses the pieces on all host threads.
//
// ReSparse (reference: resparse_spm, src/resources/python/quantify/quantify_util.py:375-403):
// per row, keep every nonzero if the smallest |v| exceeds the mean |v| of the whole (dense)
// matrix, else keep the ceil(n * keep) largest |v| (ties: the higher column first, the order of
// the reference's reversed ascending argsort).
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "acceles.h"
#include "aes_host.hpp"

namespace aes {
namespace {

struct Mapped {
  const char* p = nullptr;
  size_t n = 0;
  int fd = -1;
  ~Mapped() {
    if (p && n) munmap(const_cast<char*>(p), n);
    if (fd >= 0) close(fd);
  }
};

inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r'; }

// Lower-cased whitespace-separated words of one line.
std::vector<std::string> words_of(const char* b, const char* e) {
  std::vector<std::string> w;
  while (b < e) {
    while (b < e && (is_space(*b))) b++;
    const char* s = b;
    while (b < e && !is_space(*b)) b++;
    if (b > s) {
      std::string t(s, b);
      for (char& c : t) c = (char)std::tolower((unsigned char)c);
      w.push_back(t);
    }
  }
  return w;
}

// Parses an unsigned decimal at p (after blanks); returns false on a malformed field.
inline bool parse_u64(const char*& p, const char* e, uint64_t* out) {
  while (p < e && is_space(*p)) p++;
  auto r = std::from_chars(p, e, *out);
  if (r.ec != std::errc() || r.ptr == p) return false;
  p = r.ptr;
  return true;
}

inline bool parse_f64(const char*& p, const char* e, double* out) {
  while (p < e && is_space(*p)) p++;
  if (p < e && *p == '+') p++;
  auto r = std::from_chars(p, e, *out);
  if (r.ec != std::errc() || r.ptr == p) return false;
  p = r.ptr;
  return true;
}

}  // namespace

int read_mtx(const char* path, uint32_t flags, uint32_t* rows_out, uint32_t* cols_out,
             std::vector<uint32_t>* R, std::vector<uint32_t>* C, std::vector<float>* V) {
  Mapped m;
  m.fd = open(path, O_RDONLY);
  if (m.fd < 0) return fail(AES_ERR_INVALID, std::string("cannot open ") + path);
  struct stat st;
  if (fstat(m.fd, &st) != 0) return fail(AES_ERR_INVALID, std::string("cannot stat ") + path);
  m.n = (size_t)st.st_size;
  if (m.n == 0) return fail(AES_ERR_INVALID, "empty Matrix Market file");
  void* mp = mmap(nullptr, m.n, PROT_READ, MAP_PRIVATE, m.fd, 0);
  if (mp == MAP_FAILED) {
    m.n = 0;
    return fail(AES_ERR_INVALID, std::string("cannot map ") + path);
  }
  m.p = static_cast<const char*>(mp);
  const char* b = m.p;
  const char* end = m.p + m.n;
  auto line_end = [&](const char* s) {
    const char* q = static_cast<const char*>(memchr(s, '\n', (size_t)(end - s)));
    return q ? q : end;
  };

  // banner: %%MatrixMarket matrix coordinate <real|integer|pattern> <general|symmetric>
  const char* le = line_end(b);
  std::vector<std::string> ban = words_of(b, le);
  if (ban.size() < 5 || ban[0] != "%%matrixmarket" || ban[1] != "matrix")
    return fail(AES_ERR_INVALID, "not a Matrix Market matrix file");
  if (ban[2] != "coordinate") return fail(AES_ERR_UNSUPPORTED, "only coordinate Matrix Market files");
  const bool pattern = ban[3] == "pattern";
  if (!pattern && ban[3] != "real" && ban[3] != "integer" && ban[3] != "double")
    return fail(AES_ERR_UNSUPPORTED, "Matrix Market field must be real, integer or pattern");
  const bool symmetric = ban[4] == "symmetric";
  if (!symmetric && ban[4] != "general")
    return fail(AES_ERR_UNSUPPORTED, "Matrix Market symmetry must be general or symmetric");
  // comments, then the size line
  b = le < end ? le + 1 : end;
  while (b < end) {
    le = line_end(b);
    const char* s = b;
    while (s < le && is_space(*s)) s++;
    if (s < le && *s != '%') break;
    b = le < end ? le + 1 : end;
  }
  if (b >= end) return fail(AES_ERR_INVALID, "Matrix Market size line missing");
  uint64_t nr = 0, nc = 0, nz = 0;
  {
    const char* p = b;
    le = line_end(b);
    if (!parse_u64(p, le, &nr) || !parse_u64(p, le, &nc) || !parse_u64(p, le, &nz))
      return fail(AES_ERR_INVALID, "bad Matrix Market size line");
    b = le < end ? le + 1 : end;
  }
  if (nr == 0 || nr > 0xFFFFFFFFull || nc == 0 || nc > 0xFFFFFFFFull)
    return fail(AES_ERR_UNSUPPORTED, "Matrix Market shape out of range");

  // split the data at line boundaries and parse the pieces in parallel
  const size_t bytes = (size_t)(end - b);
  const unsigned nt = std::max(1u, std::min<unsigned>(64, (unsigned)(bytes >> 22) + 1));
  std::vector<const char*> cut(nt + 1);
  cut[0] = b;
  cut[nt] = end;
  for (unsigned t = 1; t < nt; t++) {
    const char* s = b + bytes * t / nt;
    if (s < cut[t - 1]) s = cut[t - 1];
    const char* q = line_end(s);
    cut[t] = q < end ? q + 1 : end;
  }
  struct Piece {
    std::vector<uint32_t> r, c;
    std::vector<float> v;
    std::string err;
  };
  std::vector<Piece> pc(nt);
  const bool zero = flags & AES_MTX_ZERO_INDEXED;
  parallel_for(nt, 1, [&](uint64_t t0, uint64_t t1) {
    for (uint64_t t = t0; t < t1; t++) {
      Piece& P = pc[t];
      const char* s = cut[t];
      const char* e = cut[t + 1];
      while (s < e) {
        const char* l = static_cast<const char*>(memchr(s, '\n', (size_t)(e - s)));
        if (!l) l = e;
        const char* p = s;
        while (p < l && is_space(*p)) p++;
        if (p < l && *p != '%') {
          uint64_t i = 0, j = 0;
          double v = 1.0;
          if (!parse_u64(p, l, &i) || !parse_u64(p, l, &j) || (!pattern && !parse_f64(p, l, &v))) {
            P.err = "malformed Matrix Market entry";
            return;
          }
          if (!zero) {
            if (i == 0 || j == 0) {
              P.err = "Matrix Market index 0 in a one-based file";
              return;
            }
            i--;
            j--;
          }
          if (i >= nr || j >= nc) {
            P.err = "Matrix Market index out of range";
            return;
          }
          P.r.push_back((uint32_t)i);
          P.c.push_back((uint32_t)j);
          P.v.push_back((float)v);
        }
        s = l < e ? l + 1 : e;
      }
    }
  });
  uint64_t total = 0;
  for (auto& P : pc) {
    if (!P.err.empty()) return fail(AES_ERR_INVALID, P.err);
    total += P.r.size();
  }
  if (total != nz)
    return fail(AES_ERR_INVALID, "Matrix Market file has " + std::to_string(total) +
                                     " entries, the size line says " + std::to_string(nz));
  R->clear();
  C->clear();
  V->clear();
  R->reserve(total);
  C->reserve(total);
  V->reserve(total);
  for (auto& P : pc) {
    R->insert(R->end(), P.r.begin(), P.r.end());
    C->insert(C->end(), P.c.begin(), P.c.end());
    V->insert(V->end(), P.v.begin(), P.v.end());
  }
  // symmetric files: mirror the off-diagonal entries after the stored ones (utils.hpp undirect)
  if (symmetric && !(flags & AES_MTX_KEEP_DIRECTED)) {
    const uint64_t n0 = R->size();
    for (uint64_t i = 0; i < n0; i++) {
      if ((*R)[i] != (*C)[i]) {
        if ((*C)[i] >= nr || (*R)[i] >= nc)
          return fail(AES_ERR_INVALID, "symmetric Matrix Market file with a non-square shape");
        R->push_back((*C)[i]);
        C->push_back((*R)[i]);
        V->push_back((*V)[i]);
      }
    }
  }
  if (flags & AES_MTX_SORT) {
    // (row, col) order, equal keys in file order
    std::vector<uint64_t> ord(R->size());
    for (uint64_t i = 0; i < ord.size(); i++) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](uint64_t a, uint64_t b2) {
      return (*R)[a] != (*R)[b2] ? (*R)[a] < (*R)[b2] : (*C)[a] < (*C)[b2];
    });
    std::vector<uint32_t> r2(ord.size()), c2(ord.size());
    std::vector<float> v2(ord.size());
    for (uint64_t i = 0; i < ord.size(); i++) {
      r2[i] = (*R)[ord[i]];
      c2[i] = (*C)[ord[i]];
      v2[i] = (*V)[ord[i]];
    }
    R->swap(r2);
    C->swap(c2);
    V->swap(v2);
  }
  *rows_out = (uint32_t)nr;
  *cols_out = (uint32_t)nc;
  return AES_OK;
}

int resparse(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
             uint32_t cols, double keep, std::vector<uint64_t>* optr, std::vector<uint32_t>* ocol,
             std::vector<float>* oval, double* mean_abs) {
  const uint64_t nnz = ptr[rows];
  // mean |v| over all rows x cols entries (zeros included), compensated summation per block
  const uint64_t nb = std::max<uint64_t>(1, std::min<uint64_t>(256, nnz / (1 << 16) + 1));
  std::vector<double> bs(nb, 0.0), bc(nb, 0.0);
  parallel_for(nb, 1, [&](uint64_t b0, uint64_t b1) {
    for (uint64_t bb = b0; bb < b1; bb++) {
      const uint64_t s = nnz * bb / nb, e = nnz * (bb + 1) / nb;
      double sum = 0.0, c = 0.0;
      for (uint64_t i = s; i < e; i++) {
        const double x = std::fabs((double)val[i]);
        const double t = sum + x;
        c += std::fabs(sum) >= x ? (sum - t) + x : (x - t) + sum;
        sum = t;
      }
      bs[bb] = sum;
      bc[bb] = c;
    }
  });
  double sum = 0.0, c = 0.0;
  for (uint64_t bb = 0; bb < nb; bb++) {
    for (double x : {bs[bb], bc[bb]}) {
      const double t = sum + x;
      c += std::fabs(sum) >= std::fabs(x) ? (sum - t) + x : (x - t) + sum;
      sum = t;
    }
  }
  const double avg = (sum + c) / ((double)rows * (double)cols);
  if (mean_abs) *mean_abs = avg;

  // pass 1: kept count per row; pass 2: write
  std::vector<uint64_t> kept(rows, 0);
  auto row_keep = [&](uint32_t r, std::vector<uint64_t>& idx, bool write, uint64_t out0) {
    idx.clear();
    double mn = INFINITY;
    for (uint64_t e = ptr[r]; e < ptr[r + 1]; e++) {
      if (val[e] == 0.0f) continue;  // explicit zeros are not nonzeros
      idx.push_back(e);
      mn = std::min(mn, std::fabs((double)val[e]));
    }
    const uint64_t n = idx.size();
    if (n == 0) return (uint64_t)0;
    uint64_t k = n;
    if (!(mn > avg)) {
      k = (uint64_t)std::ceil((double)n * keep);
      if (k > n) k = n;
      // largest |v| first; equal |v|: higher column first
      std::stable_sort(idx.begin(), idx.end(), [&](uint64_t a, uint64_t b2) {
        const float fa = std::fabs(val[a]), fb = std::fabs(val[b2]);
        if (fa != fb) return fa > fb;
        return col[a] > col[b2];
      });
      idx.resize(k);
      std::sort(idx.begin(), idx.end());  // back to column order
    }
    if (write) {
      for (uint64_t i = 0; i < k; i++) {
        (*ocol)[out0 + i] = col[idx[i]];
        (*oval)[out0 + i] = val[idx[i]];
      }
    }
    return k;
  };
  parallel_for(rows, 1 << 14, [&](uint64_t r0, uint64_t r1) {
    std::vector<uint64_t> idx;
    for (uint64_t r = r0; r < r1; r++) kept[r] = row_keep((uint32_t)r, idx, false, 0);
  });
  optr->assign((size_t)rows + 1, 0);
  for (uint32_t r = 0; r < rows; r++) (*optr)[r + 1] = (*optr)[r] + kept[r];
  ocol->assign((*optr)[rows], 0);
  oval->assign((*optr)[rows], 0.0f);
  parallel_for(rows, 1 << 14, [&](uint64_t r0, uint64_t r1) {
    std::vector<uint64_t> idx;
    for (uint64_t r = r0; r < r1; r++) row_keep((uint32_t)r, idx, true, (*optr)[r]);
  });
  return AES_OK;
}

}  // namespace aes

extern "C" {

int aes_read_mtx(const char* path, uint32_t flags, uint32_t* rows, uint32_t* cols, uint64_t* nnz,
                 uint32_t** row, uint32_t** col, float** val) {
  if (!path || !rows || !cols || !nnz || !row || !col || !val)
    return aes::fail(AES_ERR_INVALID, "NULL argument");
  *row = *col = nullptr;
  *val = nullptr;
  std::vector<uint32_t> R, C;
  std::vector<float> V;
  int rc = aes::read_mtx(path, flags, rows, cols, &R, &C, &V);
  if (rc) return rc;
  const size_t n = R.size();
  uint32_t* r = static_cast<uint32_t*>(std::malloc(std::max<size_t>(n, 1) * 4));
  uint32_t* c = static_cast<uint32_t*>(std::malloc(std::max<size_t>(n, 1) * 4));
  float* v = static_cast<float*>(std::malloc(std::max<size_t>(n, 1) * 4));
  if (!r || !c || !v) {
    std::free(r);
    std::free(c);
    std::free(v);
    return aes::fail(AES_ERR_NOMEM, "host allocation failed");
  }
  if (n) {
    std::memcpy(r, R.data(), n * 4);
    std::memcpy(c, C.data(), n * 4);
    std::memcpy(v, V.data(), n * 4);
  }
  *nnz = n;
  *row = r;
  *col = c;
  *val = v;
  return AES_OK;
}

void aes_free(void* p) { std::free(p); }

int aes_write_mtx(const char* path, const uint32_t* row, const uint32_t* col, const float* val,
                  uint32_t rows, uint32_t cols, uint64_t nnz, uint32_t flags) {
  if (!path || (nnz && (!row || !col || !val))) return aes::fail(AES_ERR_INVALID, "NULL argument");
  for (uint64_t i = 0; i < nnz; i++)
    if (row[i] >= rows || col[i] >= cols) return aes::fail(AES_ERR_INVALID, "index out of range");
  FILE* f = std::fopen(path, "wb");
  if (!f) return aes::fail(AES_ERR_INVALID, std::string("cannot create ") + path);
  const uint32_t base = (flags & AES_MTX_ZERO_INDEXED) ? 0 : 1;
  std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n%%\n%u %u %llu\n", rows, cols,
               (unsigned long long)nnz);
  // %.9g: every FP32 value reads back bit for bit
  std::vector<char> buf(1 << 20);
  size_t used = 0;
  for (uint64_t i = 0; i < nnz; i++) {
    if (used + 64 > buf.size()) {
      std::fwrite(buf.data(), 1, used, f);
      used = 0;
    }
    used += (size_t)std::snprintf(buf.data() + used, 64, "%u %u %.9g\n", row[i] + base,
                                  col[i] + base, (double)val[i]);
  }
  std::fwrite(buf.data(), 1, used, f);
  const bool ok = std::ferror(f) == 0;
  if (std::fclose(f) != 0 || !ok) return aes::fail(AES_ERR_INVALID, std::string("write failed: ") + path);
  return AES_OK;
}

int aes_resparse(const uint64_t* ptr, const uint32_t* col, const float* val, uint32_t rows,
                 uint32_t cols, double keep, uint64_t* out_ptr, uint32_t* out_col,
                 float* out_val, uint64_t cap, uint64_t* out_nnz) {
  if (!ptr || !out_nnz) return aes::fail(AES_ERR_INVALID, "NULL argument");
  if (rows == 0 || cols == 0) return aes::fail(AES_ERR_INVALID, "empty shape");
  if (!(keep > 0.0 && keep <= 1.0)) return aes::fail(AES_ERR_INVALID, "keep must be in (0, 1]");
  if (ptr[rows] && (!col || !val)) return aes::fail(AES_ERR_INVALID, "NULL CSR array");
  int rc = aes::check_csr(ptr, col, rows, cols);
  if (rc) return rc;
  for (uint32_t r = 0; r < rows; r++)
    for (uint64_t e = ptr[r] + 1; e < ptr[r + 1]; e++)
      if (col[e] == col[e - 1]) return aes::fail(AES_ERR_INVALID, "duplicate (row, col) entry");
  std::vector<uint64_t> op;
  std::vector<uint32_t> oc;
  std::vector<float> ov;
  rc = aes::resparse(ptr, col, val, rows, cols, keep, &op, &oc, &ov, nullptr);
  if (rc) return rc;
  *out_nnz = op[rows];
  if (out_ptr) std::memcpy(out_ptr, op.data(), ((size_t)rows + 1) * 8);
  if (out_col || out_val) {
    if (cap < op[rows]) return aes::fail(AES_ERR_INVALID, "output arrays too small");
    if (out_col && !oc.empty()) std::memcpy(out_col, oc.data(), oc.size() * 4);
    if (out_val && !ov.empty()) std::memcpy(out_val, ov.data(), ov.size() * 4);
  }
  return AES_OK;
}

}  // extern "C"
