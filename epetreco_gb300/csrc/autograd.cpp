// autograd.cpp -- the system matrix as a differentiable torch operator.
//
// A torch::autograd::Function in libtorch C++: forward y = A x (batched over
// the leading dimension of x), backward grad_x = A^T grad_y, both computed by
// libepet_gb300 -- the stored form uses the CSR and its column-major copy
// (scatter-free transpose), the matrix-free form recomputes the chords of
// every pass from the rays (epet_project_forward / epet_project_back) and
// stores nothing.  Exposed to Python as epetreco_gb300._autograd.
#include <ATen/cuda/CUDAContext.h>
#include <torch/extension.h>

#include <vector>

#include "epet_gb300.h"

namespace {

void check(epet_status s) {
  TORCH_CHECK(s == EPET_OK, "epet_gb300: ", epet_last_error());
}

epet_stream_t stream() {
  return reinterpret_cast<epet_stream_t>(at::cuda::getCurrentCUDAStream().stream());
}

void check_vec(const torch::Tensor& t, torch::ScalarType dt, const char* what) {
  TORCH_CHECK(t.is_cuda() && t.is_contiguous() && t.scalar_type() == dt, what,
              ": expected a contiguous CUDA tensor of the right type");
}

// Stored matrix: tensors of the CSR and of its column-major copy.
struct Stored {
  torch::Tensor row_ptr, col, val, col_ptr, row, cval;
  int64_t m, n;
  epet_csr csr() const {
    return epet_csr{m, n, col.numel(), row_ptr.data_ptr<int64_t>(), col.data_ptr<int32_t>(),
                    val.data_ptr<float>()};
  }
  epet_csc csc() const {
    return epet_csc{m, n, row.numel(), col_ptr.data_ptr<int64_t>(), row.data_ptr<int32_t>(),
                    cval.data_ptr<float>()};
  }
};

torch::Tensor apply_stored(const Stored& S, const torch::Tensor& x, bool trans) {
  const int64_t in = trans ? S.m : S.n, out = trans ? S.n : S.m;
  TORCH_CHECK(x.size(-1) == in, "projector: last dimension ", x.size(-1), " != ", in);
  auto xc = x.contiguous().to(torch::kFloat32);
  auto x2 = xc.reshape({-1, in});
  auto y = torch::empty({x2.size(0), out}, x2.options());
  epet_csr a = S.csr();
  epet_csc c = S.csc();
  for (int64_t b = 0; b < x2.size(0); b++)
    check(epet_csrmv(trans ? 1 : 0, &a, &c, 1.f, x2[b].data_ptr<float>(), 0.f,
                     y[b].data_ptr<float>(), stream()));
  auto shape = x.sizes().vec();
  shape.back() = out;
  return y.reshape(shape);
}

class StoredProjection : public torch::autograd::Function<StoredProjection> {
 public:
  static torch::Tensor forward(torch::autograd::AutogradContext* ctx, torch::Tensor x,
                               torch::Tensor row_ptr, torch::Tensor col, torch::Tensor val,
                               torch::Tensor col_ptr, torch::Tensor row, torch::Tensor cval,
                               int64_t n) {
    ctx->save_for_backward({row_ptr, col, val, col_ptr, row, cval});
    ctx->saved_data["n"] = n;
    Stored S{row_ptr, col, val, col_ptr, row, cval, row_ptr.numel() - 1, n};
    return apply_stored(S, x, false);
  }
  static torch::autograd::tensor_list backward(torch::autograd::AutogradContext* ctx,
                                               torch::autograd::tensor_list g) {
    auto v = ctx->get_saved_variables();
    const int64_t n = ctx->saved_data["n"].toInt();
    Stored S{v[0], v[1], v[2], v[3], v[4], v[5], v[0].numel() - 1, n};
    auto gx = apply_stored(S, g[0], true);
    return {gx, torch::Tensor(), torch::Tensor(), torch::Tensor(), torch::Tensor(),
            torch::Tensor(), torch::Tensor(), torch::Tensor()};
  }
};

// Matrix-free: the problem as a flat float64 vector of its float and int32
// fields (each exactly representable) and the 64-bit seed on its own.
epet_problem unpack(const std::vector<double>& f, int64_t seed) {
  TORCH_CHECK(f.size() == 22, "problem vector must hold 22 numbers");
  epet_problem p{};
  p.setup = epet_setup{(float)f[0], (float)f[1], (int)f[2], (int)f[3], (int)f[4], (int)f[5],
                       (int)f[6], (float)f[7], (float)f[8], (float)f[9], (float)f[10]};
  p.grid = epet_grid{{(float)f[11], (float)f[12], (float)f[13]},
                     {(float)f[14], (float)f[15], (float)f[16]},
                     {(int)f[17], (int)f[18], (int)f[19]}};
  p.nrays = (int)f[20];
  p.seed = (uint64_t)seed;
  p.ray_mode = (int32_t)f[21];
  return p;
}

torch::Tensor apply_free(const std::vector<double>& pf, int64_t seed, const torch::Tensor& rows,
                         const torch::Tensor& x, bool trans) {
  const epet_problem p = unpack(pf, seed);
  const int64_t V = (int64_t)p.grid.n[0] * p.grid.n[1] * p.grid.n[2], m = rows.numel();
  const int64_t in = trans ? m : V, out = trans ? V : m;
  TORCH_CHECK(x.size(-1) == in, "projector: last dimension ", x.size(-1), " != ", in);
  auto x2 = x.contiguous().to(torch::kFloat32).reshape({-1, in});
  auto y = trans ? torch::zeros({x2.size(0), out}, x2.options())
                 : torch::empty({x2.size(0), out}, x2.options());
  for (int64_t b = 0; b < x2.size(0); b++) {
    if (trans)
      check(epet_project_back(&p, rows.data_ptr<int32_t>(), m, x2[b].data_ptr<float>(),
                              y[b].data_ptr<float>(), 0, nullptr, 0, stream()));
    else
      check(epet_project_forward(&p, rows.data_ptr<int32_t>(), m, x2[b].data_ptr<float>(),
                                 y[b].data_ptr<float>(), 0, nullptr, 0, stream()));
  }
  auto shape = x.sizes().vec();
  shape.back() = out;
  return y.reshape(shape);
}

class FreeProjection : public torch::autograd::Function<FreeProjection> {
 public:
  static torch::Tensor forward(torch::autograd::AutogradContext* ctx, torch::Tensor x,
                               torch::Tensor rows, std::vector<double> problem, int64_t seed) {
    ctx->save_for_backward({rows});
    ctx->saved_data["problem"] = problem;
    ctx->saved_data["seed"] = seed;
    return apply_free(problem, seed, rows, x, false);
  }
  static torch::autograd::tensor_list backward(torch::autograd::AutogradContext* ctx,
                                               torch::autograd::tensor_list g) {
    auto rows = ctx->get_saved_variables()[0];
    auto pf = ctx->saved_data["problem"].toDoubleVector();
    const int64_t seed = ctx->saved_data["seed"].toInt();
    return {apply_free(pf, seed, rows, g[0], true), torch::Tensor(), torch::Tensor(),
            torch::Tensor()};
  }
};

torch::Tensor project_stored(torch::Tensor x, torch::Tensor row_ptr, torch::Tensor col,
                             torch::Tensor val, torch::Tensor col_ptr, torch::Tensor row,
                             torch::Tensor cval, int64_t n) {
  check_vec(row_ptr, torch::kInt64, "row_ptr");
  check_vec(col, torch::kInt32, "col");
  check_vec(val, torch::kFloat32, "val");
  check_vec(col_ptr, torch::kInt64, "col_ptr");
  check_vec(row, torch::kInt32, "row");
  check_vec(cval, torch::kFloat32, "cval");
  TORCH_CHECK(x.is_cuda(), "x must be a CUDA tensor");
  return StoredProjection::apply(x, row_ptr, col, val, col_ptr, row, cval, n);
}

torch::Tensor project_free(torch::Tensor x, torch::Tensor rows, std::vector<double> problem,
                           int64_t seed) {
  check_vec(rows, torch::kInt32, "rows");
  TORCH_CHECK(x.is_cuda(), "x must be a CUDA tensor");
  return FreeProjection::apply(x, rows, problem, seed);
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
  m.def("project_stored", &project_stored,
        "y = A x with the stored CSR; backward A^T g over the column-major copy");
  m.def("project_free", &project_free,
        "y = A x recomputing the chords per pass; backward A^T g likewise");
}
