// torch_ops.cpp -- libtorch operator over the C ABI: the data-consistency
// loss of one respiratory bin as a torch::autograd::Function, so that
// gradients flow to the complex64 image and to the sample coordinates (and
// from there, through differentiable PyTorch code, to wave-trajectory
// parameters).
//
//   torch.ops.cgsense.dc_loss(handle, bin, x, k, y) -> float64 scalar
//     handle  the cgs_ctx pointer of a context with coil maps and bins set
//     x       complex64 CUDA tensor, the image (img voxels, contiguous)
//     k       float64 CUDA tensor [ns][3], the coordinates of every sample
//     y       complex64 CUDA tensor [n_ch][ns], measured samples
//   L = 1/2 sum_c sum_i D_i |(E_c S_c x)_i - y_ci|^2, E_c = nufftFWD
//   (Reco.cpp:521-553).  The forward pass computes L and, for the inputs
//   that require gradients, dL/dx (as PyTorch's convention for a real loss
//   of a complex input: dL/dRe + i dL/dIm) and dL/dk in the same kernels;
//   backward scales them by the incoming gradient.
#include <torch/torch.h>
#include <torch/library.h>
#include <c10/cuda/CUDAStream.h>

#include "cgsense_c.h"

namespace {

using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

cgs_ctx* as_ctx(int64_t h) { return reinterpret_cast<cgs_ctx*>(static_cast<intptr_t>(h)); }

void check(cgs_ctx* c, int st, const char* what)
{
    TORCH_CHECK(st == CGS_OK, what, " failed (status ", st, "): ", c ? cgs_last_error(c) : "no context");
}

struct DcLoss : public torch::autograd::Function<DcLoss> {
    static torch::Tensor forward(AutogradContext* ctx, int64_t handle, int64_t bin, const torch::Tensor& x,
                                 const torch::Tensor& k, const torch::Tensor& y)
    {
        cgs_ctx* c = as_ctx(handle);
        TORCH_CHECK(c != nullptr, "dc_loss: null context");
        TORCH_CHECK(x.is_cuda() && x.scalar_type() == torch::kComplexFloat && x.is_contiguous(),
                    "dc_loss: x must be a contiguous complex64 CUDA tensor");
        TORCH_CHECK(k.is_cuda() && k.scalar_type() == torch::kFloat64 && k.is_contiguous() && k.dim() == 2 &&
                        k.size(1) == 3,
                    "dc_loss: k must be a contiguous float64 CUDA tensor [ns][3]");
        TORCH_CHECK(y.is_cuda() && y.scalar_type() == torch::kComplexFloat && y.is_contiguous(),
                    "dc_loss: y must be a contiguous complex64 CUDA tensor [n_ch][ns]");
        const bool need_x = x.requires_grad(), need_k = k.requires_grad();
        auto stream = c10::cuda::getCurrentCUDAStream(x.device().index());
        check(c, cgs_set_stream(c, stream.stream()), "cgs_set_stream");
        check(c, cgs_update_trajectory_d(c, k.data_ptr<double>()), "cgs_update_trajectory_d");
        torch::Tensor gx = need_x ? torch::empty_like(x) : torch::zeros({0}, x.options());
        torch::Tensor gk = need_k ? torch::empty({k.size(0), 3}, k.options().dtype(torch::kFloat32))
                                  : torch::zeros({0}, k.options().dtype(torch::kFloat32));
        double loss = 0.0;
        check(c, cgs_loss_grad_d(c, (int32_t)bin, x.data_ptr(), y.data_ptr(), &loss, need_x ? gx.data_ptr() : nullptr,
                                 need_k ? gk.data_ptr() : nullptr),
              "cgs_loss_grad_d");
        ctx->save_for_backward({gx, gk});
        ctx->saved_data["need_x"] = need_x;
        ctx->saved_data["need_k"] = need_k;
        return torch::full({}, loss, x.options().dtype(torch::kFloat64));
    }

    static variable_list backward(AutogradContext* ctx, variable_list g)
    {
        auto saved = ctx->get_saved_variables();
        const torch::Tensor go = g[0];
        torch::Tensor gx, gk;
        if (ctx->saved_data["need_x"].toBool()) gx = saved[0] * go.to(torch::kFloat32);
        if (ctx->saved_data["need_k"].toBool()) gk = saved[1].to(torch::kFloat64) * go;
        return {torch::Tensor(), torch::Tensor(), gx, gk, torch::Tensor()};
    }
};

torch::Tensor dc_loss(int64_t handle, int64_t bin, const torch::Tensor& x, const torch::Tensor& k,
                      const torch::Tensor& y)
{
    return DcLoss::apply(handle, bin, x, k, y);
}

}  // namespace

TORCH_LIBRARY(cgsense, m)
{
    m.def("dc_loss(int handle, int bin, Tensor x, Tensor k, Tensor y) -> Tensor", dc_loss);
}
