// minife_gb300.hpp -- header-only C++ shim over the C ABI (minife_gb300.h)
// with the reference's operator interface for the solve path.
//
// The reference (Mantevo miniFE, ref/ variant) binds this path through C++
// templates; this header keeps those types and signatures so reference-style
// host code compiles against the GB300 implementation unchanged:
//
//   CSRMatrix<S,LO,GO>   ref/src/CSRMatrix.hpp:43-129   (same fields)
//   ELLMatrix<S,LO,GO>   ref/src/ELLMatrix.hpp:41-130   (same fields; the
//                        reference built with MINIFE_ELL_MATRIX)
//   Vector<S,LO,GO>      ref/src/Vector.hpp:36-61       (same fields)
//   matvec_std<M,V>      ref/src/SparseMatrix_functions.hpp:545-578
//   matvec_and_dot       ref/src/SparseMatrix_functions.hpp:491-536
//   dot, waxpby, fused_waxpby  ref/src/Vector_functions.hpp:127-226
//   impose_dirichlet     ref/src/SparseMatrix_functions.hpp:434-480
//   write_matrix, write_vector  SparseMatrix_functions.hpp:98-140,
//                        Vector_functions.hpp:49-82 (MINIFE_DEBUG dumps)
//   cg_solve             ref/src/cg_solve.hpp:69-229
//   Box, simple_mesh_description (bc_rows_0 / bc_rows_1)
//                        ref/utils/Box.hpp, ref/src/simple_mesh_description.hpp:39-224
//   generate_matrix_structure  ref/src/generate_matrix_structure.hpp:47-149
//   assemble_FE_data, perform_element_loop
//                        ref/src/assemble_FE_data.hpp:38-73, perform_element_loop.hpp:40-104
//
// The containers stay in host std::vectors like the reference's; each call
// copies its operands to the device, runs the library's CUDA kernels and
// copies results back (cg_solve does this once for the whole solve).  Only
// Scalar = double, LocalOrdinal = GlobalOrdinal = int -- the reference's
// default build (ref/src/Makefile:3-6) -- is supported, on one rank (the
// local box is the global box).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <set>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "minife_gb300.h"

namespace minife_gb300 {

typedef double timer_type;
enum CG_TIMES { WAXPY = 0, DOT = 1, MATVEC = 2, MATVECDOT = 3, TOTAL = 4, NUM_TIMERS = 5 };

class Error : public std::runtime_error {
 public:
  Error(mfe_status s, const std::string& what)
      : std::runtime_error(what + ": " + mfe_status_string(s)), status(s) {}
  mfe_status status;
};

// Process-wide context on device 0 (one stream), created on first use.
class Context {
 public:
  static Context& get()
  {
    static Context c;
    return c;
  }
  mfe_ctx* h() { return ctx_; }
  void check(mfe_status s, const char* what)
  {
    if (s != MFE_OK) throw Error(s, std::string(what) + " (" + mfe_last_error_string(ctx_) + ")");
  }
  // device buffer cache by role, grown on demand
  void* buf(int slot, size_t bytes)
  {
    if (bytes > cap_[slot]) {
      if (ptr_[slot]) mfe_device_free(ctx_, ptr_[slot]);
      ptr_[slot] = nullptr;
      check(mfe_device_alloc(ctx_, bytes, &ptr_[slot]), "mfe_device_alloc");
      cap_[slot] = bytes;
    }
    return ptr_[slot];
  }
  ~Context()
  {
    for (int i = 0; i < kSlots; ++i)
      if (ptr_[i]) mfe_device_free(ctx_, ptr_[i]);
    mfe_ctx_destroy(ctx_);
  }

 private:
  Context()
  {
    mfe_status s = mfe_ctx_create(0, &ctx_);
    if (s != MFE_OK) throw Error(s, "mfe_ctx_create(0)");
  }
  static constexpr int kSlots = 12;
  mfe_ctx* ctx_ = nullptr;
  void* ptr_[kSlots] = {};
  size_t cap_[kSlots] = {};
};

template <typename Scalar, typename LocalOrdinal, typename GlobalOrdinal>
struct CSRMatrix {
  static_assert(std::is_same<Scalar, double>::value && std::is_same<LocalOrdinal, int>::value &&
                    std::is_same<GlobalOrdinal, int>::value,
                "minife_gb300 supports CSRMatrix<double,int,int>");
  typedef Scalar ScalarType;
  typedef LocalOrdinal LocalOrdinalType;
  typedef GlobalOrdinal GlobalOrdinalType;

  bool has_local_indices = false;
  std::vector<GlobalOrdinal> rows;
  std::vector<LocalOrdinal> row_offsets;
  std::vector<LocalOrdinal> row_offsets_external;
  std::vector<GlobalOrdinal> packed_cols;
  std::vector<Scalar> packed_coefs;
  LocalOrdinal num_cols = 0;

  size_t num_nonzeros() const { return row_offsets.empty() ? 0 : row_offsets.back(); }
  void reserve_space(unsigned nrows, unsigned ncols_per_row)
  {
    rows.resize(nrows);
    row_offsets.resize(nrows + 1);
    packed_cols.reserve((size_t)nrows * ncols_per_row);
    packed_coefs.reserve((size_t)nrows * ncols_per_row);
  }
  // one rank: rows[i] == i, so the row pointer is a direct index
  void get_row_pointers(GlobalOrdinal row, size_t& row_length, GlobalOrdinal*& cols,
                        Scalar*& coefs)
  {
    if (row < 0 || (size_t)row + 1 >= row_offsets.size()) {
      row_length = 0;
      return;
    }
    const LocalOrdinal off = row_offsets[row];
    row_length = (size_t)(row_offsets[row + 1] - off);
    cols = &packed_cols[off];
    coefs = &packed_coefs[off];
  }
};

// ELLMatrix: num_cols_per_row entries per row, row-major, each row's
// columns ascending and then padding with column 0, value 0
// (MatrixInitOp<ELLMatrix>, MatrixInitOp.hpp:160-220)
template <typename Scalar, typename LocalOrdinal, typename GlobalOrdinal>
struct ELLMatrix {
  static_assert(std::is_same<Scalar, double>::value && std::is_same<LocalOrdinal, int>::value &&
                    std::is_same<GlobalOrdinal, int>::value,
                "minife_gb300 supports ELLMatrix<double,int,int>");
  typedef Scalar ScalarType;
  typedef LocalOrdinal LocalOrdinalType;
  typedef GlobalOrdinal GlobalOrdinalType;

  bool has_local_indices = false;
  std::vector<GlobalOrdinal> rows;
  std::vector<GlobalOrdinal> cols;
  std::vector<Scalar> coefs;
  LocalOrdinal num_cols = 0;
  LocalOrdinal num_cols_per_row = 0;

  size_t num_nonzeros() const { return rows.size() * (size_t)num_cols_per_row; }
  void reserve_space(unsigned nrows, unsigned ncols_per_row)
  {
    rows.resize(nrows);
    cols.resize((size_t)nrows * ncols_per_row);
    coefs.resize((size_t)nrows * ncols_per_row);
    num_cols_per_row = (LocalOrdinal)ncols_per_row;
  }
  // one rank: rows[i] == i.  The row's length ends at its last entry with a
  // nonzero column, as the reference's (ELLMatrix.hpp:122-128): the padding
  // after it has column 0
  void get_row_pointers(GlobalOrdinal row, size_t& row_length, GlobalOrdinal*& cols_ptr,
                        Scalar*& coefs_ptr)
  {
    if (row < 0 || (size_t)row >= rows.size()) {
      row_length = 0;
      return;
    }
    cols_ptr = &cols[(size_t)row * num_cols_per_row];
    coefs_ptr = &coefs[(size_t)row * num_cols_per_row];
    int idx = num_cols_per_row - 1;
    while (idx >= 0 && cols_ptr[idx] == 0) --idx;
    row_length = (size_t)(idx + 1);
  }
};

template <typename Scalar, typename LocalOrdinal, typename GlobalOrdinal>
struct Vector {
  typedef Scalar ScalarType;
  typedef LocalOrdinal LocalOrdinalType;
  typedef GlobalOrdinal GlobalOrdinalType;
  Vector(GlobalOrdinal startIdx, LocalOrdinal local_sz)
      : startIndex(startIdx), local_size(local_sz), coefs(local_sz, 0.0) {}
  GlobalOrdinal startIndex;
  LocalOrdinal local_size;
  std::vector<Scalar> coefs;
};

namespace detail {
enum { SLOT_RO = 0, SLOT_COLS, SLOT_VALS, SLOT_X, SLOT_Y, SLOT_W, SLOT_ROWS, SLOT_X2, SLOT_Y2,
       SLOT_W2 };

inline void h2d(void* d, const void* h, size_t bytes)
{
  Context& c = Context::get();
  c.check(mfe_memcpy_h2d(c.h(), d, h, bytes), "mfe_memcpy_h2d");
}
inline void d2h(void* h, const void* d, size_t bytes)
{
  Context& c = Context::get();
  c.check(mfe_memcpy_d2h(c.h(), h, d, bytes), "mfe_memcpy_d2h");
}

template <typename M>
mfe_csr upload(const M& A)
{
  Context& c = Context::get();
  mfe_csr m;
  std::memset(&m, 0, sizeof(m));
  m.nrows = (int64_t)A.rows.size();
  m.ncols = m.nrows;
  m.nnz = (int64_t)A.packed_cols.size();
  m.dtype = MFE_F64;
  m.row_offsets = static_cast<int32_t*>(c.buf(SLOT_RO, 4 * (size_t)(m.nrows + 1)));
  m.cols = static_cast<int32_t*>(c.buf(SLOT_COLS, 4 * (size_t)(m.nnz + 4)));
  m.vals = c.buf(SLOT_VALS, 8 * (size_t)(m.nnz + 4));
  h2d(m.row_offsets, A.row_offsets.data(), 4 * (size_t)(m.nrows + 1));
  h2d(m.cols, A.packed_cols.data(), 4 * (size_t)m.nnz);
  h2d(m.vals, A.packed_coefs.data(), 8 * (size_t)m.nnz);
  return m;
}

template <typename S, typename LO, typename GO>
mfe_ell upload_ell(const ELLMatrix<S, LO, GO>& A)
{
  Context& c = Context::get();
  mfe_ell e;
  std::memset(&e, 0, sizeof(e));
  e.nrows = (int64_t)A.rows.size();
  e.ncols_per_row = A.num_cols_per_row;
  e.dtype = MFE_F64;
  const size_t ne = A.rows.size() * (size_t)A.num_cols_per_row;
  e.cols = static_cast<int32_t*>(c.buf(SLOT_COLS, 4 * ne + 16));
  e.vals = c.buf(SLOT_VALS, 8 * ne + 16);
  h2d(e.cols, A.cols.data(), 4 * ne);
  h2d(e.vals, A.coefs.data(), 8 * ne);
  return e;
}

// an ELL matrix's device CSR (from mfe_csr m) converted in the shim's ELL
// buffers and copied into A: columns when structure, always the values
template <typename S, typename LO, typename GO>
void download_ell(const mfe_csr& m, ELLMatrix<S, LO, GO>& A, bool structure)
{
  Context& c = Context::get();
  const int K = 27;
  const size_t ne = (size_t)m.nrows * K;
  mfe_ell e;
  std::memset(&e, 0, sizeof(e));
  e.ncols_per_row = K;
  e.cols = static_cast<int32_t*>(c.buf(SLOT_X2, 4 * ne + 16));
  e.vals = c.buf(SLOT_Y2, 8 * ne + 16);
  c.check(mfe_csr_to_ell(c.h(), &m, &e), "mfe_csr_to_ell");
  if (structure) {
    A.rows.resize((size_t)m.nrows);
    for (int64_t i = 0; i < m.nrows; ++i) A.rows[(size_t)i] = (int)i;
    A.cols.resize(ne);
    d2h(A.cols.data(), e.cols, 4 * ne);
    A.num_cols_per_row = K;
    A.has_local_indices = true;
    A.num_cols = (int)m.nrows;
  }
  A.coefs.resize(ne);
  d2h(A.coefs.data(), e.vals, 8 * ne);
}
}  // namespace detail

// matvec_std<CSR>: y = A x (SparseMatrix_functions.hpp:548-577)
template <typename MatrixType, typename VectorType>
struct matvec_std {
  void operator()(MatrixType& A, VectorType& x, VectorType& y)
  {
    Context& c = Context::get();
    mfe_csr m = detail::upload(A);
    const size_t n = A.rows.size();
    double* dx = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
    double* dy = static_cast<double*>(c.buf(detail::SLOT_Y, 8 * n + 16));
    detail::h2d(dx, x.coefs.data(), 8 * n);
    c.check(mfe_spmv(c.h(), &m, dx, dy), "mfe_spmv");
    detail::d2h(y.coefs.data(), dy, 8 * n);
  }
};

// matvec_std<ELLMatrix> (SparseMatrix_functions.hpp:579-611): every stored
// entry, the padding adding 0 * x[0]
template <typename S, typename LO, typename GO, typename VectorType>
struct matvec_std<ELLMatrix<S, LO, GO>, VectorType> {
  void operator()(ELLMatrix<S, LO, GO>& A, VectorType& x, VectorType& y)
  {
    Context& c = Context::get();
    mfe_ell e = detail::upload_ell(A);
    const size_t n = A.rows.size();
    double* dx = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
    double* dy = static_cast<double*>(c.buf(detail::SLOT_Y, 8 * n + 16));
    detail::h2d(dx, x.coefs.data(), 8 * n);
    c.check(mfe_spmv_ell(c.h(), &e, dx, dy), "mfe_spmv_ell");
    detail::d2h(y.coefs.data(), dy, 8 * n);
  }
};

template <typename MatrixType, typename VectorType>
void matvec(MatrixType& A, VectorType& x, VectorType& y)
{
  matvec_std<MatrixType, VectorType>()(A, x, y);
}

template <typename MatrixType, typename VectorType>
double matvec_and_dot(MatrixType& A, VectorType& x, VectorType& y)
{
  Context& c = Context::get();
  mfe_csr m = detail::upload(A);
  const size_t n = A.rows.size();
  double* dx = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
  double* dy = static_cast<double*>(c.buf(detail::SLOT_Y, 8 * n + 16));
  detail::h2d(dx, x.coefs.data(), 8 * n);
  double r = 0;
  c.check(mfe_matvec_and_dot(c.h(), &m, dx, dy, &r), "mfe_matvec_and_dot");
  detail::d2h(y.coefs.data(), dy, 8 * n);
  return r;
}

// dot (Vector_functions.hpp:194-226)
template <typename VectorType>
double dot(const VectorType& x, const VectorType& y)
{
  Context& c = Context::get();
  const size_t n = x.coefs.size();
  double* dx = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
  double* dy = static_cast<double*>(c.buf(detail::SLOT_Y, 8 * n + 16));
  detail::h2d(dx, x.coefs.data(), 8 * n);
  detail::h2d(dy, y.coefs.data(), 8 * n);
  double r = 0;
  c.check(mfe_dot(c.h(), (int64_t)n, dx, dy, &r), "mfe_dot");
  return r;
}

// waxpby (Vector_functions.hpp:127-150): w = alpha x + beta y
template <typename VectorType>
void waxpby(double alpha, const VectorType& x, double beta, const VectorType& y, VectorType& w)
{
  Context& c = Context::get();
  const size_t n = x.coefs.size();
  double* dx = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
  double* dy = static_cast<double*>(c.buf(detail::SLOT_Y, 8 * n + 16));
  double* dw = static_cast<double*>(c.buf(detail::SLOT_W, 8 * n + 16));
  detail::h2d(dx, x.coefs.data(), 8 * n);
  detail::h2d(dy, y.coefs.data(), 8 * n);
  c.check(mfe_waxpby(c.h(), (int64_t)n, alpha, dx, beta, dy, dw), "mfe_waxpby");
  detail::d2h(w.coefs.data(), dw, 8 * n);
}

// fused_waxpby (Vector_functions.hpp:154-185): both updates in one pass
template <typename VectorType>
void fused_waxpby(double alpha, const VectorType& x, double beta, const VectorType& y,
                  VectorType& w, double alpha2, const VectorType& x2, double beta2,
                  const VectorType& y2, VectorType& w2)
{
  Context& c = Context::get();
  const size_t n = x.coefs.size();
  double* d[6];
  const int slots[6] = {detail::SLOT_X, detail::SLOT_Y, detail::SLOT_W,
                        detail::SLOT_X2, detail::SLOT_Y2, detail::SLOT_W2};
  for (int i = 0; i < 6; ++i) d[i] = static_cast<double*>(c.buf(slots[i], 8 * n + 16));
  detail::h2d(d[0], x.coefs.data(), 8 * n);
  detail::h2d(d[1], y.coefs.data(), 8 * n);
  detail::h2d(d[3], x2.coefs.data(), 8 * n);
  detail::h2d(d[4], y2.coefs.data(), 8 * n);
  c.check(mfe_fused_waxpby(c.h(), (int64_t)n, alpha, d[0], beta, d[1], d[2], alpha2, d[3], beta2,
                           d[4], d[5]),
          "mfe_fused_waxpby");
  detail::d2h(w.coefs.data(), d[2], 8 * n);
  detail::d2h(w2.coefs.data(), d[5], 8 * n);
}

// impose_dirichlet (SparseMatrix_functions.hpp:434-480)
template <typename MatrixType, typename VectorType>
void impose_dirichlet(double prescribed_value, MatrixType& A, VectorType& b, int /*global_nx*/,
                      int /*global_ny*/, int /*global_nz*/, const std::set<int>& bc_rows)
{
  Context& c = Context::get();
  mfe_csr m = detail::upload(A);
  const size_t n = A.rows.size();
  double* db = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
  detail::h2d(db, b.coefs.data(), 8 * n);
  std::vector<int32_t> rows(bc_rows.begin(), bc_rows.end());  // std::set is ascending
  int32_t* drows = static_cast<int32_t*>(c.buf(detail::SLOT_ROWS, 4 * rows.size() + 16));
  if (!rows.empty()) detail::h2d(drows, rows.data(), 4 * rows.size());
  c.check(mfe_impose_dirichlet(c.h(), &m, db, prescribed_value, drows, (int64_t)rows.size()),
          "mfe_impose_dirichlet");
  detail::d2h(A.packed_coefs.data(), m.vals, 8 * A.packed_coefs.size());
  detail::d2h(b.coefs.data(), db, 8 * n);
}

// impose_dirichlet for the ELLMatrix: the rows as get_row_pointers gives
// them (the padding left out) go through the same device kernel as a CSR,
// and the values come back into the ELL rows
template <typename S, typename LO, typename GO, typename VectorType>
void impose_dirichlet(double prescribed_value, ELLMatrix<S, LO, GO>& A, VectorType& b,
                      int global_nx, int global_ny, int global_nz, const std::set<int>& bc_rows)
{
  CSRMatrix<S, LO, GO> C;
  const size_t n = A.rows.size();
  C.rows = A.rows;
  C.row_offsets.assign(n + 1, 0);
  std::vector<size_t> len(n);
  for (size_t r = 0; r < n; ++r) {
    GO* cp = nullptr;
    S* vp = nullptr;
    A.get_row_pointers((GO)r, len[r], cp, vp);
    C.row_offsets[r + 1] = C.row_offsets[r] + (LO)len[r];
    C.packed_cols.insert(C.packed_cols.end(), cp, cp + len[r]);
    C.packed_coefs.insert(C.packed_coefs.end(), vp, vp + len[r]);
  }
  impose_dirichlet(prescribed_value, C, b, global_nx, global_ny, global_nz, bc_rows);
  const size_t K = (size_t)A.num_cols_per_row;
  for (size_t r = 0; r < n; ++r)
    std::copy(C.packed_coefs.begin() + C.row_offsets[r], C.packed_coefs.begin() + C.row_offsets[r + 1],
              A.coefs.begin() + r * K);
}

// write_matrix / write_vector (SparseMatrix_functions.hpp:98-140,
// Vector_functions.hpp:49-82; MINIFE_DEBUG), one rank: "<filename>.1.0"
// holding "nrows nnz" (nnz = num_nonzeros(), the ELL's padded count) and one
// "row col coef" line per entry of each row as get_row_pointers gives it, or
// "n" and one "index coef" line per entry; the default std::ostream number
// format.  The containers are on the host, so these only format them.
template <typename MatrixType>
void write_matrix(const std::string& filename, MatrixType& mat)
{
  std::ofstream ofs((filename + ".1.0").c_str());
  if (!ofs) throw Error(MFE_BAD_ARG, "write_matrix: cannot open " + filename + ".1.0");
  ofs << mat.rows.size() << " " << mat.num_nonzeros() << std::endl;
  for (size_t i = 0; i < mat.rows.size(); ++i) {
    size_t len = 0;
    typename MatrixType::GlobalOrdinalType* cols = nullptr;
    typename MatrixType::ScalarType* coefs = nullptr;
    mat.get_row_pointers(mat.rows[i], len, cols, coefs);
    for (size_t j = 0; j < len; ++j) ofs << mat.rows[i] << " " << cols[j] << " " << coefs[j] << std::endl;
  }
}

template <typename VectorType>
void write_vector(const std::string& filename, const VectorType& vec)
{
  std::ofstream ofs((filename + ".1.0").c_str());
  if (!ofs) throw Error(MFE_BAD_ARG, "write_vector: cannot open " + filename + ".1.0");
  ofs << vec.local_size << std::endl;
  for (size_t i = 0; i < (size_t)vec.local_size; ++i)
    ofs << vec.startIndex + (typename VectorType::GlobalOrdinalType)i << " " << vec.coefs[i] << std::endl;
}

// ---- the assembly side, one rank ----

// Box (ref/utils/Box.hpp): three [lo, hi) element ranges, box[d][0..1]
struct Box {
  int ranges[6];
  int* operator[](int xyz) { return &ranges[xyz * 2]; }
  const int* operator[](int xyz) const { return &ranges[xyz * 2]; }
};

// simple_mesh_description (simple_mesh_description.hpp:39-224) for one rank:
// the global box and the two Dirichlet row sets -- bc_rows_0 (faces x = 0,
// y = 0, z = 0, y = 1, z = 1) and bc_rows_1 (face x = 1) -- from the
// library (mfe_box_bc_rows).  The local box must be the global box.
template <typename GlobalOrdinal>
class simple_mesh_description {
 public:
  simple_mesh_description(const Box& global_box_in, const Box& local_box_in)
      : global_box(global_box_in), local_box(local_box_in)
  {
    for (int d = 0; d < 3; ++d)
      if (global_box[d][0] != 0 || local_box[d][0] != global_box[d][0] ||
          local_box[d][1] != global_box[d][1] || global_box[d][1] < 1)
        throw Error(MFE_NOT_SUPPORTED, "simple_mesh_description: one rank, boxes from 0");
    Context& c = Context::get();
    const int nx = global_box[0][1], ny = global_box[1][1], nz = global_box[2][1];
    for (int which = 0; which < 2; ++which) {
      int64_t cnt = 0;
      c.check(mfe_box_bc_rows(c.h(), nx, ny, nz, which, nullptr, &cnt), "mfe_box_bc_rows");
      std::vector<int32_t> rows((size_t)cnt);
      if (cnt > 0) {
        int32_t* dr = static_cast<int32_t*>(c.buf(detail::SLOT_ROWS, 4 * (size_t)cnt + 16));
        c.check(mfe_box_bc_rows(c.h(), nx, ny, nz, which, dr, &cnt), "mfe_box_bc_rows");
        detail::d2h(rows.data(), dr, 4 * (size_t)cnt);
      }
      std::set<GlobalOrdinal>& dst = which == 0 ? bc_rows_0 : bc_rows_1;
      dst.insert(rows.begin(), rows.end());
    }
  }
  Box global_box;
  Box local_box;
  std::set<GlobalOrdinal> bc_rows_0;
  std::set<GlobalOrdinal> bc_rows_1;
};

namespace detail {
// the device CSR of the mesh's box in the shim's buffers (structure only,
// or with the element loop's values and b)
inline mfe_csr box_csr(int nx, int ny, int nz)
{
  Context& c = Context::get();
  int64_t n = 0, nnz = 0;
  c.check(mfe_box_dims(nx, ny, nz, &n, &nnz), "mfe_box_dims");
  mfe_csr m;
  std::memset(&m, 0, sizeof(m));
  m.nrows = n;
  m.ncols = n;
  m.nnz = nnz;
  m.dtype = MFE_F64;
  m.row_offsets = static_cast<int32_t*>(c.buf(SLOT_RO, 4 * (size_t)(n + 1)));
  m.cols = static_cast<int32_t*>(c.buf(SLOT_COLS, 4 * (size_t)(nnz + 4)));
  m.vals = c.buf(SLOT_VALS, 8 * (size_t)(nnz + 4));
  return m;
}

template <typename M>
void download(const mfe_csr& m, M& A, bool structure)
{
  if (structure) {
    A.rows.resize((size_t)m.nrows);
    for (int64_t i = 0; i < m.nrows; ++i) A.rows[(size_t)i] = (int)i;
    A.row_offsets.resize((size_t)m.nrows + 1);
    A.packed_cols.resize((size_t)m.nnz);
    d2h(A.row_offsets.data(), m.row_offsets, 4 * (size_t)(m.nrows + 1));
    d2h(A.packed_cols.data(), m.cols, 4 * (size_t)m.nnz);
    A.has_local_indices = true;
    A.num_cols = (int)m.nrows;
  }
  A.packed_coefs.resize((size_t)m.nnz);
  d2h(A.packed_coefs.data(), m.vals, 8 * (size_t)m.nnz);
}
}  // namespace detail

// generate_matrix_structure (generate_matrix_structure.hpp:47-149,
// MatrixInitOp.hpp:127-156): rows, row offsets and ascending 27-point
// columns of the mesh's box, coefficients zero.  Returns 0.
template <typename GlobalOrdinal, typename MatrixType>
int generate_matrix_structure(const simple_mesh_description<GlobalOrdinal>& mesh, MatrixType& A)
{
  Context& c = Context::get();
  const int nx = mesh.global_box[0][1], ny = mesh.global_box[1][1], nz = mesh.global_box[2][1];
  mfe_csr m = detail::box_csr(nx, ny, nz);
  c.check(mfe_generate_structure(c.h(), nx, ny, nz, &m), "mfe_generate_structure");
  detail::download(m, A, true);
  return 0;
}

// generate_matrix_structure for the ELLMatrix (MatrixInitOp.hpp:160-220):
// 27 entries per row, each row's columns ascending, then column 0 padding
template <typename GlobalOrdinal, typename S, typename LO, typename GO>
int generate_matrix_structure(const simple_mesh_description<GlobalOrdinal>& mesh,
                              ELLMatrix<S, LO, GO>& A)
{
  Context& c = Context::get();
  const int nx = mesh.global_box[0][1], ny = mesh.global_box[1][1], nz = mesh.global_box[2][1];
  mfe_csr m = detail::box_csr(nx, ny, nz);
  c.check(mfe_generate_structure(c.h(), nx, ny, nz, &m), "mfe_generate_structure");
  detail::download_ell(m, A, true);
  return 0;
}

// perform_element_loop (perform_element_loop.hpp:40-104) over the whole
// box: every element's diffusion matrix and source vector summed into A
// (whose structure generate_matrix_structure made) and b, in element
// order; params is accepted for signature compatibility.
template <typename GlobalOrdinal, typename MatrixType, typename VectorType, typename Params>
void perform_element_loop(const simple_mesh_description<GlobalOrdinal>& mesh, const Box& box,
                          MatrixType& A, VectorType& b, Params& /*params*/)
{
  for (int d = 0; d < 3; ++d)
    if (box[d][0] != mesh.local_box[d][0] || box[d][1] != mesh.local_box[d][1])
      throw Error(MFE_NOT_SUPPORTED, "perform_element_loop: the element box is the local box");
  Context& c = Context::get();
  const int nx = mesh.global_box[0][1], ny = mesh.global_box[1][1], nz = mesh.global_box[2][1];
  mfe_csr m = detail::box_csr(nx, ny, nz);
  if (A.row_offsets.size() != (size_t)m.nrows + 1 || A.packed_cols.size() != (size_t)m.nnz)
    throw Error(MFE_BAD_ARG, "perform_element_loop: A lacks the box's structure");
  double* db = static_cast<double*>(c.buf(detail::SLOT_X, 8 * (size_t)m.nrows + 16));
  c.check(mfe_assemble(c.h(), nx, ny, nz, nullptr, &m, db, 0), "mfe_assemble");
  detail::download(m, A, false);
  b.coefs.resize((size_t)m.nrows);
  detail::d2h(b.coefs.data(), db, 8 * (size_t)m.nrows);
}

// perform_element_loop for the ELLMatrix: the same element sums, held in the
// ELL rows (A's structure from generate_matrix_structure)
template <typename GlobalOrdinal, typename S, typename LO, typename GO, typename VectorType,
          typename Params>
void perform_element_loop(const simple_mesh_description<GlobalOrdinal>& mesh, const Box& box,
                          ELLMatrix<S, LO, GO>& A, VectorType& b, Params& /*params*/)
{
  for (int d = 0; d < 3; ++d)
    if (box[d][0] != mesh.local_box[d][0] || box[d][1] != mesh.local_box[d][1])
      throw Error(MFE_NOT_SUPPORTED, "perform_element_loop: the element box is the local box");
  Context& c = Context::get();
  const int nx = mesh.global_box[0][1], ny = mesh.global_box[1][1], nz = mesh.global_box[2][1];
  mfe_csr m = detail::box_csr(nx, ny, nz);
  if (A.rows.size() != (size_t)m.nrows || A.num_cols_per_row != 27 ||
      A.cols.size() != (size_t)m.nrows * 27)
    throw Error(MFE_BAD_ARG, "perform_element_loop: A lacks the box's ELL structure");
  c.check(mfe_generate_structure(c.h(), nx, ny, nz, &m), "mfe_generate_structure");
  double* db = static_cast<double*>(c.buf(detail::SLOT_X, 8 * (size_t)m.nrows + 16));
  c.check(mfe_assemble(c.h(), nx, ny, nz, nullptr, &m, db, 0), "mfe_assemble");
  detail::download_ell(m, A, false);
  b.coefs.resize((size_t)m.nrows);
  detail::d2h(b.coefs.data(), db, 8 * (size_t)m.nrows);
}

// assemble_FE_data (assemble_FE_data.hpp:38-73): the element loop over the
// local box; the Dirichlet conditions follow with impose_dirichlet, as in
// the reference's driver (driver.hpp:214-218)
template <typename GlobalOrdinal, typename MatrixType, typename VectorType, typename Params>
void assemble_FE_data(const simple_mesh_description<GlobalOrdinal>& mesh, MatrixType& A,
                      VectorType& b, Params& params)
{
  perform_element_loop(mesh, mesh.local_box, A, b, params);
}

// cg_solve (cg_solve.hpp:69-229).  The Matvec argument is accepted for
// signature compatibility; the solve always uses the library's kernels.
template <typename OperatorType, typename VectorType, typename Matvec>
void cg_solve(OperatorType& A, const VectorType& b, VectorType& x, Matvec /*matvec*/,
              typename OperatorType::LocalOrdinalType max_iter, double& tolerance,
              typename OperatorType::LocalOrdinalType& num_iters, double& normr,
              timer_type* my_cg_times)
{
  Context& c = Context::get();
  mfe_cg_opts o;
  mfe_cg_opts_default(&o);
  o.max_iter = max_iter;
  o.tol = tolerance;
  mfe_cg_result r;
  const mfe_status s = mfe_cg_solve_host(
      c.h(), (int64_t)A.rows.size(), (int64_t)A.packed_cols.size(), A.row_offsets.data(),
      A.packed_cols.data(), A.packed_coefs.data(), b.coefs.data(), x.coefs.data(), &o, &r);
  if (s == MFE_BREAKDOWN) {
    // the reference reports breakdown on std::cerr and returns (cg_solve.hpp:188)
  } else if (s != MFE_OK && s != MFE_MAXITER) {
    c.check(s, "mfe_cg_solve_host");
  }
  num_iters = r.num_iters;
  normr = r.normr;
  if (my_cg_times)
    for (int t = 0; t < NUM_TIMERS; ++t) my_cg_times[t] = r.times[t];
}

// cg_solve with the ELLMatrix (the reference built with MINIFE_ELL_MATRIX):
// the library's ELL CG (mfe_cg_solve_ell)
template <typename S, typename LO, typename GO, typename VectorType, typename Matvec>
void cg_solve(ELLMatrix<S, LO, GO>& A, const VectorType& b, VectorType& x, Matvec /*matvec*/,
              LO max_iter, double& tolerance, LO& num_iters, double& normr,
              timer_type* my_cg_times)
{
  Context& c = Context::get();
  mfe_ell e = detail::upload_ell(A);
  const size_t n = A.rows.size();
  double* db = static_cast<double*>(c.buf(detail::SLOT_X, 8 * n + 16));
  double* dx = static_cast<double*>(c.buf(detail::SLOT_Y, 8 * n + 16));
  detail::h2d(db, b.coefs.data(), 8 * n);
  detail::h2d(dx, x.coefs.data(), 8 * n);
  mfe_cg_opts o;
  mfe_cg_opts_default(&o);
  o.max_iter = max_iter;
  o.tol = tolerance;
  mfe_cg_result r;
  const mfe_status s = mfe_cg_solve_ell(c.h(), &e, db, dx, &o, &r);
  if (s == MFE_BREAKDOWN) {
    // the reference reports breakdown on std::cerr and returns (cg_solve.hpp:188)
  } else if (s != MFE_OK && s != MFE_MAXITER) {
    c.check(s, "mfe_cg_solve_ell");
  }
  detail::d2h(x.coefs.data(), dx, 8 * n);
  num_iters = r.num_iters;
  normr = r.normr;
  if (my_cg_times)
    for (int t = 0; t < NUM_TIMERS; ++t) my_cg_times[t] = r.times[t];
}

}  // namespace minife_gb300
