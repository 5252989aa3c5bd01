// sf_unet.h -- the learned solver's 3D U-Net on the GPU (host interface).
//
// Architecture (4 levels, 16/32/64/64 channels, 3x3x3 convolutions, ReLU, additive skips, 1x1 head):
//   E0: c(16->16) c(16->16) = s0 | E1: pool c(16->32) c(32->32) = s1 | E2: pool c(32->64) c(64->64) = s2
//   E3: pool c(64->64) c(64->64) | D2: up+s2 c(64->64) c(64->32) | D1: up+s1 c(32->32) c(32->16)
//   D0: up+s0 c(16->16) c(16->16) | head 1x1 (16->1)
// Input: 16 feature channels per cell (BF16), output: one FP32 value per cell.  Parameters are FP32 master
// copies (flat, layer by layer: weights [tap][cout][cin] then bias [cout]) with BF16 copies for the kernels.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "sf_internal.cuh"

namespace sf {

struct ConvLayer {
    int cin, cout, level, taps;
    long long woff, boff;  // offsets into the flat parameter vector
    long long wbf;         // offset into the BF16 weight copies
};

class UNet {
   public:
    static constexpr int kCin = 16;
    explicit UNet(cudaStream_t st);
    ~UNet();

    long long num_params() const { return nparams_; }
    const std::vector<ConvLayer> &layers() const { return layers_; }
    cudaError_t set_params(const float *host);
    cudaError_t get_params(float *host);
    cudaError_t get_grads(float *host);

    // out[v] = net(features)[v]; features BF16 [n][16] on the device.  training = false (inference: out must be
    // given) runs in a workspace whose decoder reuses the encoder's dead buffers and holds no gradients, about a
    // quarter of the training workspace; a backward pass needs a training forward first.
    cudaError_t forward(const Dims &d, const __nv_bfloat16 *features, float *out, bool training = true);
    // gradients of sum(dout * out) w.r.t. the parameters (after a forward on the same features)
    cudaError_t backward(const Dims &d, const float *dout);
    // one Adam step on the cosine loss 1 - (o.t)^2 / (|o|^2 |t|^2); returns the loss before the step
    cudaError_t train_step(const Dims &d, const __nv_bfloat16 *features, const float *target, float lr, double &loss);

    // the 16 input channels of a system in face-coefficient form (FP64 fine level) with rhs b
    cudaError_t features(const Dims &d, const Coef<double> &cf, const double *b, __nv_bfloat16 *feat);
    // active cells (D > 0) counted by the last features()
    double active_cells() const { return active_; }
    // channel 0 of existing features set to r * inv_rms (FP32 r on the cells), the other channels unchanged
    cudaError_t set_rhs_channel(const Dims &d, const float *r, double inv_rms, __nv_bfloat16 *feat);
    float *output() { return out_; }
    // convolution kernels: 0 warp-level MMA (mma.sync) throughout; 1 (default) tcgen05 + TMA for the forward,
    // input-gradient and weight-gradient convolutions; 2 tcgen05 for the weight gradient alone (the rest as mode 0)
    void set_mode(int m) { mode_ = m; }
    int mode() const { return mode_; }
    long long tc_launches() const { return tc_launches_; }
    // reads (and clears) the device error flag of the tcgen05 kernels; synchronises the stream
    cudaError_t check_device_errors();

    std::string last_error;

   private:
    cudaError_t ensure(const Dims &d, bool training);
    cudaError_t ensure_wgrad_ws();
    void conv_fwd(const ConvLayer &L, const Dims &d, const __nv_bfloat16 *x, __nv_bfloat16 *y);
    void conv_bwd(const ConvLayer &L, const Dims &d, const __nv_bfloat16 *x, const __nv_bfloat16 *post,
                  const float *dpost, float *dx /* nullable */);
    void refresh_bf16();
    void *alloc(size_t bytes);

    cudaStream_t st_;
    std::vector<ConvLayer> layers_;
    long long nparams_ = 0, nbf_ = 0;
    float *p_ = nullptr, *g_ = nullptr, *m1_ = nullptr, *m2_ = nullptr;
    __nv_bfloat16 *wb_ = nullptr, *wt_ = nullptr;  // forward weights, mirrored/transposed for input gradients
    __nv_bfloat16 *wbp_ = nullptr, *wtp_ = nullptr;  // the same with taps ordered by z shift (64-long z lines)
    long long step_ = 0;
    std::vector<void *> persist_;
    // per-grid workspace
    Dims dims_[4]{};
    bool have_ws_ = false, ws_training_ = false;
    std::vector<void *> ws_;
    __nv_bfloat16 *A0a, *S0, *P1, *A1a, *S1, *P2, *A2a, *S2, *P3, *A3a, *A3b, *U2, *D2a, *D2b, *U1, *D1a, *D1b, *U0,
        *D0a, *D0b;
    const __nv_bfloat16 *feat_ = nullptr;
    float *gA[4], *gB[4], *gU[3];
    __nv_bfloat16 *gbf[4];
    __nv_bfloat16 *wg_dy_ = nullptr, *wg_x_ = nullptr;  // channel-major copies for the tcgen05 weight gradient
    float *out_ = nullptr, *dout_ = nullptr, *wpart_ = nullptr, *hpart_ = nullptr;
    double *dots_ = nullptr, *dots_host_ = nullptr, *redpart_ = nullptr;
    long long wpart_elems_ = 0;
    int mode_ = 1;
    double active_ = 0;
    int *err_ = nullptr;
    long long tc_launches_ = 0;
};

}  // namespace sf
