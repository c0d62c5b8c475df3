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

#include <map>

#include "cgsense_c.h"

namespace {

using torch::autograd::AutogradContext;
using torch::autograd::variable_list;

cgs_ctx* as_ctx(int64_t h) { return reinterpret_cast<cgs_ctx*>(static_cast<intptr_t>(h)); }

void check(cgs_ctx* c, int st, const char* what)
{
    TORCH_CHECK(st == CGS_OK, what, " failed (status ", st, "): ", c ? cgs_last_error(c) : "no context");
}

// The context keeps one trajectory; uploading it marks the spreading lists
// stale (a host rebuild at the next spreading call), so the k last uploaded
// by these operators is not uploaded again while it is unchanged: same
// tensor (held here, so its storage cannot be reused), same version, and no
// other trajectory set on the context since (its serial number).
struct SeenK {
    torch::Tensor k;
    int64_t version = -1;
    uint64_t serial = 0;
};
std::map<cgs_ctx*, SeenK>& seen_k()
{
    static std::map<cgs_ctx*, SeenK> m;
    return m;
}

void use_trajectory(cgs_ctx* c, const torch::Tensor& k)
{
    TORCH_CHECK(k.is_cuda() && k.scalar_type() == torch::kFloat64 && k.is_contiguous() && k.dim() == 2 &&
                    k.size(1) == 3,
                "k must be a contiguous float64 CUDA tensor [ns][3]");
    SeenK& s = seen_k()[c];
    if (s.k.defined() && s.k.is_same(k) && s.version == k._version() && s.serial == cgs_trajectory_serial(c)) return;
    check(c, cgs_update_trajectory_d(c, k.data_ptr<double>()), "cgs_update_trajectory_d");
    s.k = k;
    s.version = k._version();
    s.serial = cgs_trajectory_serial(c);
}

// Orders the library's work after PyTorch's pending work on the current
// stream and PyTorch's later work after the library's: an event on each
// side (the context keeps its own stream and its captured graphs).
struct StreamJoin {
    cudaStream_t ts = nullptr, cs = nullptr;
    StreamJoin(cgs_ctx* c, const torch::Tensor& t)
    {
        ts = c10::cuda::getCurrentCUDAStream(t.device().index()).stream();
        cs = static_cast<cudaStream_t>(cgs_get_stream(c));
        if (cs != ts) wait(cs, ts);
    }
    ~StreamJoin()
    {
        if (cs != ts) wait(ts, cs);
    }
    static void wait(cudaStream_t waiter, cudaStream_t producer)
    {
        cudaEvent_t e;
        TORCH_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess, "cudaEventCreate failed");
        cudaEventRecord(e, producer);
        cudaStreamWaitEvent(waiter, e, 0);
        cudaEventDestroy(e);
    }
};

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
        StreamJoin join(c, x);
        use_trajectory(c, k);
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

void check_images(const torch::Tensor& t, const char* what)
{
    TORCH_CHECK(t.is_cuda() && t.scalar_type() == torch::kComplexFloat && t.is_contiguous(), what,
                " must be a contiguous complex64 CUDA tensor [nb][image]");
}

// q = A(k) p for bins [bin0, bin0 + nb), A = sum_c conj(S_c) E_c^H D E_c S_c
// (Reco.cpp:232-262).  Backward: dL/dp = A v (A is Hermitian),
// dL/dk = d/dk Re<v, A(k) p>.
struct ApplyA : public torch::autograd::Function<ApplyA> {
    static torch::Tensor forward(AutogradContext* ctx, int64_t handle, int64_t bin0, int64_t nb,
                                 const torch::Tensor& p, const torch::Tensor& k)
    {
        cgs_ctx* c = as_ctx(handle);
        check_images(p, "p");
        StreamJoin join(c, p);
        use_trajectory(c, k);
        torch::Tensor q = torch::empty_like(p);
        check(c, cgs_apply_ehde_d(c, (int32_t)bin0, (int32_t)nb, reinterpret_cast<const float*>(p.data_ptr()),
                                  reinterpret_cast<float*>(q.data_ptr())),
              "cgs_apply_ehde_d");
        ctx->save_for_backward({p, k});
        ctx->saved_data["handle"] = handle;
        ctx->saved_data["bin0"] = bin0;
        ctx->saved_data["nb"] = nb;
        return q;
    }

    static variable_list backward(AutogradContext* ctx, variable_list g)
    {
        auto saved = ctx->get_saved_variables();
        const torch::Tensor p = saved[0], k = saved[1];
        cgs_ctx* c = as_ctx(ctx->saved_data["handle"].toInt());
        const int32_t bin0 = (int32_t)ctx->saved_data["bin0"].toInt(), nb = (int32_t)ctx->saved_data["nb"].toInt();
        const torch::Tensor v = g[0].contiguous();
        torch::Tensor gp, gk;
        // needs_input_grad counts the tensor inputs only: p is 0, k is 1
        if (ctx->needs_input_grad(0)) gp = torch::empty_like(v);
        if (ctx->needs_input_grad(1)) gk = torch::zeros({k.size(0), 3}, k.options().dtype(torch::kFloat32));
        {
            StreamJoin join(c, v);   // PyTorch's later work (the conversion below) waits for these
            use_trajectory(c, k);
            if (gp.defined())
                check(c, cgs_apply_ehde_d(c, bin0, nb, reinterpret_cast<const float*>(v.data_ptr()),
                                          reinterpret_cast<float*>(gp.data_ptr())),
                      "cgs_apply_ehde_d");
            if (gk.defined())
                check(c, cgs_apply_vjp_k_d(c, bin0, nb, p.data_ptr(), v.data_ptr(), gk.data_ptr()), "cgs_apply_vjp_k_d");
        }
        return {torch::Tensor(), torch::Tensor(), torch::Tensor(), gp, gk.defined() ? gk.to(torch::kFloat64) : gk};
    }
};

// b = sum_c conj(S_c) E_c^H (D y_c) for bins [bin0, bin0 + nb) (CGSense.cpp:226-235);
// backward: dL/dk = d/dk Re<v, b(k)> (y is data: no gradient).
struct Rhs : public torch::autograd::Function<Rhs> {
    static torch::Tensor forward(AutogradContext* ctx, int64_t handle, int64_t bin0, int64_t nb,
                                 const torch::Tensor& y, const torch::Tensor& k, int64_t nimg)
    {
        cgs_ctx* c = as_ctx(handle);
        TORCH_CHECK(y.is_cuda() && y.scalar_type() == torch::kComplexFloat && y.is_contiguous(),
                    "y must be a contiguous complex64 CUDA tensor [n_ch][ns]");
        torch::Tensor b = torch::empty({nb, nimg}, y.options());
        StreamJoin join(c, y);
        use_trajectory(c, k);
        check(c, cgs_rhs_d(c, (int32_t)bin0, (int32_t)nb, y.data_ptr(), b.data_ptr()), "cgs_rhs_d");
        ctx->save_for_backward({y, k});
        ctx->saved_data["handle"] = handle;
        ctx->saved_data["bin0"] = bin0;
        ctx->saved_data["nb"] = nb;
        return b;
    }

    static variable_list backward(AutogradContext* ctx, variable_list g)
    {
        auto saved = ctx->get_saved_variables();
        const torch::Tensor y = saved[0], k = saved[1];
        cgs_ctx* c = as_ctx(ctx->saved_data["handle"].toInt());
        const int32_t bin0 = (int32_t)ctx->saved_data["bin0"].toInt(), nb = (int32_t)ctx->saved_data["nb"].toInt();
        const torch::Tensor v = g[0].contiguous();
        torch::Tensor gk;
        if (ctx->needs_input_grad(1)) {   // tensor inputs: y is 0, k is 1
            gk = torch::zeros({k.size(0), 3}, k.options().dtype(torch::kFloat32));
            StreamJoin join(c, v);   // ends before the conversion below
            use_trajectory(c, k);
            check(c, cgs_rhs_vjp_k_d(c, bin0, nb, y.data_ptr(), v.data_ptr(), gk.data_ptr()), "cgs_rhs_vjp_k_d");
        }
        return {torch::Tensor(), torch::Tensor(), torch::Tensor(), torch::Tensor(),
                gk.defined() ? gk.to(torch::kFloat64) : gk, torch::Tensor()};
    }
};

torch::Tensor apply_a(int64_t handle, int64_t bin0, int64_t nb, const torch::Tensor& p, const torch::Tensor& k)
{
    return ApplyA::apply(handle, bin0, nb, p, k);
}

torch::Tensor rhs(int64_t handle, int64_t bin0, int64_t nb, const torch::Tensor& y, const torch::Tensor& k,
                  int64_t nimg)
{
    return Rhs::apply(handle, bin0, nb, y, k, nimg);
}

void forget(int64_t handle) { seen_k().erase(as_ctx(handle)); }

}  // namespace

TORCH_LIBRARY(cgsense, m)
{
    m.def("dc_loss(int handle, int bin, Tensor x, Tensor k, Tensor y) -> Tensor", dc_loss);
    m.def("apply_a(int handle, int bin0, int nb, Tensor p, Tensor k) -> Tensor", apply_a);
    m.def("rhs(int handle, int bin0, int nb, Tensor y, Tensor k, int nimg) -> Tensor", rhs);
    m.def("forget(int handle) -> ()", forget);
}
