// Gradients of the clustering energy behind a libtorch autograd function.
//
// For a fixed clustering (the engine's current labels), ClusteringEnergy maps vertex
// positions xyz (N x 3) and per-vertex densities rho (N, the metric's indicator:
// weight = dual area * rho^gradation; optional) to the total energy sum_k E_k and the
// quadric-placed cluster vertices c_k (K x 3) of vtkQEMetricForClustering
// (DiscreteRemeshing/vtkQEMetricForClustering.h:194-208 energy, :268-285 placement) or
// vtkIsotropicMetricForClustering.  Forward and backward call acvd_adjoint_on_stream
// (include/acvd_gpu.h) on torch's current CUDA stream: the backward recomputes the
// cluster sums (nothing per item is kept between the passes), the incoming energy
// cotangent stays on the device, and neither pass waits on the host.  The adjoint
// kernels run in FP64; inputs of another floating type are converted on the device
// and the gradients are returned in the inputs' types.
//
// The C ABI is reached through function pointers that bind() takes from the
// library instance the Python package has loaded (libacvd_gb300.so), so this module
// does not link against it.
#include <torch/extension.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>

#include "../../include/acvd_gpu.h"

namespace {

using torch::Tensor;
using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

using AdjointFn = decltype(&acvd_adjoint_on_stream);
using LastErrorFn = decltype(&acvd_last_error);
AdjointFn g_adjoint = nullptr;
LastErrorFn g_last_error = nullptr;

void bind(int64_t adjoint_fn, int64_t last_error_fn) {
    g_adjoint = reinterpret_cast<AdjointFn>(adjoint_fn);
    g_last_error = reinterpret_cast<LastErrorFn>(last_error_fn);
}

int adjoint(acvd_ctx* ctx, void* stream, const double* xyz, const double* rho, double gradation, const double* gE,
            const double* gC, double* energy, double* cent, double* gx, double* gr) {
    TORCH_CHECK(g_adjoint != nullptr, "acvd_adjoint_torch: bind() was not called");
    return g_adjoint(ctx, stream, xyz, rho, gradation, gE, gC, energy, nullptr, cent, gx, gr);
}

void check(int rc, acvd_ctx* ctx, const char* what) {
    TORCH_CHECK(rc == ACVD_OK, what, " failed (status ", rc, "): ", g_last_error ? g_last_error(ctx) : "");
}

const double* dptr(const Tensor& t) { return t.defined() ? t.data_ptr<double>() : nullptr; }
double* dptr_mut(Tensor& t) { return t.defined() ? t.data_ptr<double>() : nullptr; }

struct ClusteringEnergy : public torch::autograd::Function<ClusteringEnergy> {
    static variable_list forward(AutogradContext* actx, Tensor xyz, Tensor rho, int64_t engine, double gradation,
                                 int64_t k) {
        TORCH_CHECK(xyz.is_cuda() && xyz.dim() == 2 && xyz.size(1) == 3, "xyz must be a CUDA (N, 3) tensor");
        TORCH_CHECK(!rho.defined() || (rho.is_cuda() && rho.numel() == xyz.size(0)), "rho must be a CUDA (N,) tensor");
        const c10::cuda::CUDAGuard guard(xyz.device());
        acvd_ctx* ctx = reinterpret_cast<acvd_ctx*>(engine);
        Tensor x64 = xyz.detach().to(torch::kFloat64).contiguous();
        Tensor r64 = rho.defined() ? rho.detach().to(torch::kFloat64).contiguous() : Tensor();
        auto opts = x64.options();
        Tensor energy = torch::empty({}, opts);
        Tensor cent = torch::empty({k, 3}, opts);
        check(adjoint(ctx, c10::cuda::getCurrentCUDAStream(xyz.device().index()).stream(), x64.data_ptr<double>(),
                      dptr(r64), gradation, nullptr, nullptr, energy.data_ptr<double>(), cent.data_ptr<double>(),
                      nullptr, nullptr),
              ctx, "acvd_adjoint_on_stream (forward)");
        actx->save_for_backward({x64, r64});
        actx->saved_data["engine"] = engine;
        actx->saved_data["gradation"] = gradation;
        actx->saved_data["x_dtype"] = xyz.scalar_type();
        actx->saved_data["r_dtype"] = rho.defined() ? rho.scalar_type() : torch::kFloat64;
        return {energy, cent};
    }

    static variable_list backward(AutogradContext* actx, variable_list grads) {
        auto saved = actx->get_saved_variables();
        Tensor x64 = saved[0], r64 = saved[1];
        const c10::cuda::CUDAGuard guard(x64.device());
        acvd_ctx* ctx = reinterpret_cast<acvd_ctx*>(actx->saved_data["engine"].toInt());
        const double gradation = actx->saved_data["gradation"].toDouble();
        Tensor gE = grads[0].defined() ? grads[0].to(torch::kFloat64).contiguous() : Tensor();
        Tensor gC = grads[1].defined() ? grads[1].to(torch::kFloat64).contiguous() : Tensor();
        Tensor gx = torch::empty_like(x64);
        Tensor gr = r64.defined() ? torch::empty_like(r64) : Tensor();
        check(adjoint(ctx, c10::cuda::getCurrentCUDAStream(x64.device().index()).stream(), x64.data_ptr<double>(),
                      dptr(r64), gradation, dptr(gE), dptr(gC), nullptr, nullptr, gx.data_ptr<double>(),
                      dptr_mut(gr)),
              ctx, "acvd_adjoint_on_stream (backward)");
        Tensor gx_out = gx.to(actx->saved_data["x_dtype"].toScalarType());
        Tensor gr_out = gr.defined() ? gr.to(actx->saved_data["r_dtype"].toScalarType()) : Tensor();
        return {gx_out, gr_out, Tensor(), Tensor(), Tensor()};
    }
};

// (energy, centroids) of the engine's fixed clustering; engine = the acvd_ctx pointer
std::vector<Tensor> clustering_energy(Tensor xyz, c10::optional<Tensor> rho, int64_t engine, double gradation,
                                      int64_t k) {
    return ClusteringEnergy::apply(xyz, rho.has_value() ? *rho : Tensor(), engine, gradation, k);
}

}  // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.def("bind", &bind, "Function pointers of acvd_adjoint_on_stream and acvd_last_error (C ABI)");
    m.def("clustering_energy", &clustering_energy,
          "Energy and placed cluster vertices of a fixed clustering, differentiable in xyz and rho");
}
