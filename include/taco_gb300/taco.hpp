// taco's user-facing C++ API for the three statements libtacogb implements, header-only, over
// the C ABI in taco_gb300.h.  Code written against taco's API for these statements —
//
//   Format csr({Dense, Sparse});
//   Tensor<double> A("A", {m, n}, csr), x("x", {n}, Format({Dense})), y("y", {m}, Format({Dense}));
//   A.insert({i, j}, v); ... A.pack();
//   IndexVar i, j;
//   y(i) = A(i, j) * x(j);
//   y.compile(); y.assemble(); y.compute();
//
// — compiles unchanged against this header (namespace taco) and runs on the GPU.  Mirrors:
// Format / ModeFormat (include/taco/format.h; CSR = {Dense, Sparse}, src/format.cpp:393-406),
// Tensor<T> insert/pack/compile/assemble/compute/evaluate/at (include/taco/tensor.h,
// src/tensor.cpp:295-463, 605-850), IndexVar and index expressions (include/taco/index_notation/
// index_notation.h).  Statements outside the three patterns throw: taco itself would generate
// code for them.
//
// pack() follows taco's semantics: coordinates are sorted and duplicates summed
// (src/tensor.cpp:295-463).  Errors are reported by exceptions carrying tacogb_last_error().
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "taco_gb300.h"

namespace taco {

// ------------------------------------------------------------------ formats ----------------

class ModeFormat {
 public:
  enum Kind { DenseKind, CompressedKind };
  constexpr ModeFormat(Kind k = DenseKind) : kind_(k) {}
  Kind kind() const { return kind_; }
  bool operator==(const ModeFormat& o) const { return kind_ == o.kind_; }
  bool operator!=(const ModeFormat& o) const { return kind_ != o.kind_; }

 private:
  Kind kind_;
};

constexpr ModeFormat Dense(ModeFormat::DenseKind);
constexpr ModeFormat Compressed(ModeFormat::CompressedKind);
constexpr ModeFormat Sparse(ModeFormat::CompressedKind);

class Format {
 public:
  Format() = default;
  Format(const ModeFormat& m) : modes_{m}, ordering_{0} {}
  Format(std::vector<ModeFormat> modes) : modes_(std::move(modes)) {
    ordering_.resize(modes_.size());
    std::iota(ordering_.begin(), ordering_.end(), 0);
  }
  Format(std::vector<ModeFormat> modes, std::vector<int> ordering)
      : modes_(std::move(modes)), ordering_(std::move(ordering)) {
    if (ordering_.size() != modes_.size()) throw std::invalid_argument("format ordering size");
  }
  int getOrder() const { return (int)modes_.size(); }
  const std::vector<ModeFormat>& getModeFormats() const { return modes_; }
  const std::vector<int>& getModeOrdering() const { return ordering_; }
  bool operator==(const Format& o) const { return modes_ == o.modes_ && ordering_ == o.ordering_; }
  bool operator!=(const Format& o) const { return !(*this == o); }

 private:
  std::vector<ModeFormat> modes_;
  std::vector<int> ordering_;
};

inline const Format CSR({Dense, Sparse}, {0, 1});
inline const Format CSC({Dense, Sparse}, {1, 0});
inline const Format DCSR({Sparse, Sparse}, {0, 1});

// ------------------------------------------------------------------ index notation ---------

class IndexVar {
 public:
  IndexVar() : id_(next()) {}
  explicit IndexVar(const std::string& name) : id_(next()), name_(name) {}
  int id() const { return id_; }
  const std::string& getName() const { return name_; }
  bool operator==(const IndexVar& o) const { return id_ == o.id_; }
  bool operator!=(const IndexVar& o) const { return id_ != o.id_; }

 private:
  static int next() {
    static std::atomic<int> n{0};
    return n++;
  }
  int id_;
  std::string name_;
};

namespace detail {

struct TensorContent;

struct AccessNode {
  std::shared_ptr<TensorContent> tensor;
  std::vector<IndexVar> vars;
};

// The right-hand side forms the library recognises: a product of two accesses.
struct MulNode {
  AccessNode a, b;
};

inline void check(int rc, const char* what) {
  if (rc != 0)
    throw std::runtime_error(std::string(what) + " failed: " + tacogb_last_error());
}

enum class Pattern { None, SpMV, SpMM, SpGEMM };

// Owns a taco_tensor_t plus the small arrays it points to.
struct TacoStruct {
  taco_tensor_t t{};
  std::vector<int32_t> dims, ordering;
  std::vector<taco_mode_t> types;
  std::vector<uint8_t**> per_mode;
  std::vector<std::vector<uint8_t*>> slots;
  std::vector<int32_t> dense_size;  // the one-element dimension arrays of dense modes
  double fill = 0.0;
};

struct TensorContent {
  std::string name;
  std::vector<int> dims;
  Format format;
  int csize = 64;
  // coordinate buffer for insert()
  std::vector<std::vector<int>> coords;
  std::vector<double> coord_vals;
  // packed storage: CSR (pos, crd) for {Dense,Sparse}; dense values otherwise
  std::vector<int32_t> pos, crd;
  std::vector<uint8_t> vals;  // csize/8 bytes per value
  // results produced by the library are owned through these (malloc'd by libtacogb)
  void* owned_pos = nullptr;
  void* owned_crd = nullptr;
  void* owned_vals = nullptr;
  int64_t owned_nnz = 0;
  bool packed = false;
  // assignment
  bool has_assignment = false;
  std::vector<IndexVar> lhs_vars;
  MulNode rhs;
  Pattern pattern = Pattern::None;
  TacoStruct st;

  ~TensorContent() {
    std::free(owned_pos);
    std::free(owned_crd);
    std::free(owned_vals);
  }

  bool isCSR() const {
    return format.getOrder() == 2 && format.getModeFormats()[0] == Dense &&
           format.getModeFormats()[1] == Sparse && format.getModeOrdering()[0] == 0;
  }
  bool isDense() const {
    for (auto& m : format.getModeFormats())
      if (m != Dense) return false;
    return format.getOrder() < 2 || format.getModeOrdering()[0] == 0;
  }
  size_t esize() const { return (size_t)csize / 8; }

  const int32_t* posPtr() const { return owned_pos ? (const int32_t*)owned_pos : pos.data(); }
  const int32_t* crdPtr() const { return owned_crd ? (const int32_t*)owned_crd : crd.data(); }
  uint8_t* valsPtr() { return owned_vals ? (uint8_t*)owned_vals : vals.data(); }
  int64_t nnz() const {
    if (!isCSR()) {
      int64_t n = 1;
      for (int d : dims) n *= d;
      return n;
    }
    return owned_pos ? ((const int32_t*)owned_pos)[dims[0]] : (int64_t)crd.size();
  }

  // taco_tensor_t over the current storage (TensorStorage conversion layout,
  // src/storage/storage.cpp:127-177).
  taco_tensor_t* build() {
    const int order = format.getOrder();
    st = TacoStruct();
    st.dims.assign(dims.begin(), dims.end());
    st.ordering.assign(format.getModeOrdering().begin(), format.getModeOrdering().end());
    st.dense_size.resize(order);
    st.slots.resize(order);
    for (int m = 0; m < order; m++) {
      const bool sparse = format.getModeFormats()[m] == Sparse;
      st.types.push_back(sparse ? taco_mode_sparse : taco_mode_dense);
      if (sparse) {
        st.slots[m] = {(uint8_t*)posPtr(), (uint8_t*)crdPtr()};
      } else {
        st.dense_size[m] = dims[m];
        st.slots[m] = {(uint8_t*)&st.dense_size[m]};
      }
    }
    for (int m = 0; m < order; m++) st.per_mode.push_back(st.slots[m].data());
    st.t.order = order;
    st.t.dimensions = st.dims.data();
    st.t.csize = csize;
    st.t.mode_ordering = st.ordering.data();
    st.t.mode_types = st.types.data();
    st.t.indices = st.per_mode.data();
    st.t.vals = (owned_vals || !vals.empty()) ? valsPtr() : nullptr;
    st.t.fill_value = (uint8_t*)&st.fill;
    st.t.vals_size = 0;
    return &st.t;
  }

  // Takes ownership of the result arrays assemble() wrote into the struct (malloc'd by
  // libtacogb for host operands, as taco's generated assemble mallocs them).
  void adopt() {
    if (isCSR()) {
      std::free(owned_pos);
      std::free(owned_crd);
      owned_pos = (void*)st.slots[1][0];
      owned_crd = (void*)st.slots[1][1];
      pos.clear();
      crd.clear();
    }
    std::free(owned_vals);
    owned_vals = (void*)st.t.vals;
    vals.clear();
  }
};

}  // namespace detail

template <typename T> class Tensor;

class Access {
 public:
  Access(std::shared_ptr<detail::TensorContent> t, std::vector<IndexVar> vars)
      : node_{std::move(t), std::move(vars)} {}
  const detail::AccessNode& node() const { return node_; }

  struct Product {
    detail::MulNode mul;
  };
  friend Product operator*(const Access& a, const Access& b) { return Product{{a.node_, b.node_}}; }

  // `result(i, ...) = A(i, j) * B(j, ...)`: records the statement on the result tensor
  // (TensorBase assignment, src/tensor.cpp:521-545).
  void operator=(const Product& p) {
    auto& c = *node_.tensor;
    c.has_assignment = true;
    c.lhs_vars = node_.vars;
    c.rhs = p.mul;
    c.pattern = detail::Pattern::None;
  }

 private:
  detail::AccessNode node_;
};

template <typename T>
class Tensor {
  static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value,
                "libtacogb computes in double or float");

 public:
  Tensor(std::vector<int> dims, Format format) : Tensor("", std::move(dims), std::move(format)) {}
  Tensor(std::string name, std::vector<int> dims, Format format)
      : c_(std::make_shared<detail::TensorContent>()) {
    if ((int)dims.size() != format.getOrder())
      throw std::invalid_argument("tensor order does not match its format");
    c_->name = std::move(name);
    c_->dims = std::move(dims);
    c_->format = std::move(format);
    c_->csize = 8 * (int)sizeof(T);
  }

  const std::string& getName() const { return c_->name; }
  const std::vector<int>& getDimensions() const { return c_->dims; }
  int getDimension(int m) const { return c_->dims[m]; }
  const Format& getFormat() const { return c_->format; }
  int getOrder() const { return (int)c_->dims.size(); }

  void insert(const std::vector<int>& coord, T value) {
    if ((int)coord.size() != getOrder()) throw std::invalid_argument("coordinate arity");
    for (int m = 0; m < getOrder(); m++)
      if (coord[m] < 0 || coord[m] >= c_->dims[m]) throw std::out_of_range("coordinate");
    c_->coords.push_back(coord);
    c_->coord_vals.push_back((double)value);
    c_->packed = false;
  }

  // Sort the coordinates, sum duplicates and build the format's arrays.
  void pack() {
    auto& c = *c_;
    std::vector<size_t> idx(c.coords.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return c.coords[a] < c.coords[b]; });
    if (c.isCSR()) {
      const int rows = c.dims[0];
      c.pos.assign(rows + 1, 0);
      c.crd.clear();
      std::vector<T> v;
      for (size_t q = 0; q < idx.size(); q++) {
        const auto& x = c.coords[idx[q]];
        const T val = (T)c.coord_vals[idx[q]];
        if (!c.crd.empty() && q > 0 && c.coords[idx[q - 1]] == x) {
          v.back() += val;
          continue;
        }
        c.crd.push_back(x[1]);
        v.push_back(val);
        c.pos[x[0] + 1]++;
      }
      for (int i = 0; i < rows; i++) c.pos[i + 1] += c.pos[i];
      c.vals.resize(v.size() * sizeof(T));
      if (!v.empty()) std::memcpy(c.vals.data(), v.data(), c.vals.size());
    } else if (c.isDense()) {
      int64_t n = 1;
      for (int d : c.dims) n *= d;
      std::vector<T> v((size_t)n, T(0));
      for (size_t q : idx) {
        int64_t lin = 0;
        for (int m = 0; m < getOrder(); m++) lin = lin * c.dims[m] + c.coords[q][m];
        v[(size_t)lin] += (T)c.coord_vals[q];
      }
      c.vals.resize(v.size() * sizeof(T));
      std::memcpy(c.vals.data(), v.data(), c.vals.size());
    } else {
      throw std::invalid_argument("libtacogb stores CSR and dense row-major tensors");
    }
    std::free(c.owned_pos);
    std::free(c.owned_crd);
    std::free(c.owned_vals);
    c.owned_pos = c.owned_crd = c.owned_vals = nullptr;
    c.coords.clear();
    c.coord_vals.clear();
    c.packed = true;
  }

  template <typename... V>
  Access operator()(const V&... vars) {
    return Access(c_, std::vector<IndexVar>{vars...});
  }

  // Recognises the statement and binds it to libtacogb's kernels (stands for taco's
  // TensorBase::compile, src/tensor.cpp:605-674).
  void compile() {
    auto& c = *c_;
    if (!c.has_assignment) throw std::logic_error("compile(): tensor has no assignment");
    const auto& A = *c.rhs.a.tensor;
    const auto& B = *c.rhs.b.tensor;
    const auto& va = c.rhs.a.vars;
    const auto& vb = c.rhs.b.vars;
    const auto& vr = c.lhs_vars;
    const bool ij_jk = va.size() == 2 && vb.size() >= 1 && va[1] == vb[0] && !vr.empty() &&
                       vr[0] == va[0];
    if (!ij_jk || !A.isCSR()) throw unsupported();
    if (vb.size() == 1 && vr.size() == 1 && B.isDense() && c.isDense())
      c.pattern = detail::Pattern::SpMV;
    else if (vb.size() == 2 && vr.size() == 2 && vr[1] == vb[1] && B.isDense() && c.isDense())
      c.pattern = detail::Pattern::SpMM;
    else if (vb.size() == 2 && vr.size() == 2 && vr[1] == vb[1] && B.isCSR() && c.isCSR())
      c.pattern = detail::Pattern::SpGEMM;
    else
      throw unsupported();
  }

  void assemble() { run(false); }
  void compute() { run(true); }
  void evaluate() {
    compile();
    assemble();
    compute();
  }

  // Value at a coordinate (zero when not stored), as taco's Tensor<T>::at.
  T at(const std::vector<int>& coord) const {
    auto& c = *c_;
    if ((int)coord.size() != getOrder()) throw std::invalid_argument("coordinate arity");
    if (coord.size() == 2 && c.isCSR()) {
      const int32_t* p = c.posPtr();
      const int32_t* k = c.crdPtr();
      const T* v = (const T*)c.valsPtr();
      for (int32_t q = p[coord[0]]; q < p[coord[0] + 1]; q++)
        if (k[q] == coord[1]) return v[q];
      return T(0);
    }
    int64_t lin = 0;
    for (int m = 0; m < getOrder(); m++) lin = lin * c.dims[m] + coord[m];
    return ((const T*)c.valsPtr())[lin];
  }

  // Raw storage (CSR: pos/crd per row; values in storage order).
  const int32_t* pos() const { return c_->posPtr(); }
  const int32_t* crd() const { return c_->crdPtr(); }
  const T* vals() const { return (const T*)c_->valsPtr(); }
  int64_t nnz() const { return c_->nnz(); }

 private:
  std::runtime_error unsupported() const {
    return std::runtime_error("taco_gb300 implements y(i)=A(i,j)*x(j) and C(i,k)=A(i,j)*B(j,k) "
                              "with A CSR; taco generates code for '" + c_->name + "'");
  }

  void run(bool compute) {
    auto& c = *c_;
    if (c.pattern == detail::Pattern::None) compile();
    auto& A = *c.rhs.a.tensor;
    auto& B = *c.rhs.b.tensor;
    if (!A.packed && !A.coords.empty()) throw std::logic_error("operand A is not packed");
    if (!B.packed && !B.coords.empty()) throw std::logic_error("operand B is not packed");
    taco_tensor_t* ta = A.build();
    taco_tensor_t* tb = B.build();
    if (!compute) {
      taco_tensor_t* tc = c.build();
      tc->vals = nullptr;
      int rc = 0;
      switch (c.pattern) {
        case detail::Pattern::SpMV: rc = tacogb_spmv_assemble(tc, ta, tb); break;
        case detail::Pattern::SpMM: rc = tacogb_spmm_assemble(tc, ta, tb); break;
        case detail::Pattern::SpGEMM: rc = tacogb_spgemm_assemble(tc, ta, tb); break;
        default: break;
      }
      detail::check(rc, "assemble");
      c.adopt();
      c.packed = true;
      return;
    }
    taco_tensor_t* tc = c.build();
    int rc = 0;
    switch (c.pattern) {
      case detail::Pattern::SpMV: rc = tacogb_spmv_compute(tc, ta, tb); break;
      case detail::Pattern::SpMM: rc = tacogb_spmm_compute(tc, ta, tb); break;
      case detail::Pattern::SpGEMM: rc = tacogb_spgemm_compute(tc, ta, tb); break;
      default: break;
    }
    detail::check(rc, "compute");
  }

  std::shared_ptr<detail::TensorContent> c_;
};

}  // namespace taco
