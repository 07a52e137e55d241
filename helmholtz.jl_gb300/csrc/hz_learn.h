// Learned coarse-grid correction: network object and the launch helpers the
// solver uses to feed it (implemented in hz_learn.cu).
#pragma once

#include <cuda_bf16.h>

#include "hz_kernels.cuh"

namespace hz {

// 2D convolutional encoder-decoder (BF16 weights and activations, FP32
// accumulation on the tensor cores) that maps a normalised coarse residual and
// the medium to the normalised coarse error.
//   input  x [B][N][4] FP32: Re r/s, Im r/s, w^2 m h^2, gamma / w   (s = RMS of r)
//   output y [B][N][8] FP32: Re, Im of e / (h^2 s) in channels 0, 1
// N = nx * ny nodes, axis 1 (nx) fastest; nx - 1 and ny - 1 divisible by 8.
// Weights exchanged with the host are FP32, layer after layer, each layer
// [cout][9][cin] with tap t = 3 * (dy + 1) + (dx + 1).
class CoarseNet {
 public:
  static constexpr int kLayers = 8;
  explicit CoarseNet(unsigned seed);
  ~CoarseNet();
  CoarseNet(const CoarseNet&) = delete;
  CoarseNet& operator=(const CoarseNet&) = delete;

  static long long num_params();
  static bool supports(long long nx, long long ny);
  static void layer_shape(int l, int* cin, int* cout);

  void get_weights(float* host) const;
  void set_weights(const float* host);
  void get_grad(float* host) const;
  // versioned binary file: weights and the Adam state (moments, step), so that
  // training resumes where it stopped; load checks the format and the shapes
  void save(const char* path) const;
  void load(const char* path);
  // header check of a saved file without a GPU: returns 0 and the parameter
  // count and Adam step, or a negative code (-1 unreadable, -2 not a network
  // file, -3 other version, -4 other layer shapes, -5 truncated)
  static int file_info(const char* path, long long* nparams, long long* step);

  // forward pass on c.stream; x4 on the device; result in output(); train keeps
  // the activations and allocates their gradients for backward()
  void forward(Ctx& c, const float* x4, int nx, int ny, int B, bool train = false);
  const float* output() const { return y32_; }
  float* input_staging(int nx, int ny, int B);  // [B][N][4] FP32 buffer the solver packs into
  float* scale_staging(int B);                  // per-sample scale factors
  // loss and weight gradient after forward(); t [B][N][2] FP32 on the device
  double backward(Ctx& c, const float* t, int nx, int ny, int B);
  void adam(Ctx& c, double lr);
  // Adam steps over nsamples pairs (device x [S][N][4], t [S][N][2]) in shuffled
  // mini-batches; epoch-mean losses into loss_hist (host, epochs entries)
  void train(Ctx& c, const float* x, const float* t, int nx, int ny, long long nsamples, int batch, int epochs,
             double lr, unsigned seed, double* loss_hist);

  Ctx ctx;  // own stream and launch table (training, standalone inference)

  // convolution kernels: 0 = warp-level MMA (mma.sync); 1 = 5th-generation
  // tensor cores (tcgen05.mma, TMEM accumulator, operands staged by TMA) where
  // the channel counts suit it; 2 (the default) = per layer the faster of the
  // two: the tensor cores for every such layer of this network
  void set_conv_path(int path);
  int conv_path() const { return conv_path_; }
  // true when a tensor-core convolution gave up waiting (device flag; synchronous read)
  bool tc_failed();

 private:
  void conv(Ctx& c, const char* name, int nx, int ny, int B, int Cin, const __nv_bfloat16* in, int ldi, int i_off,
            int Cout, const __nv_bfloat16* w, __nv_bfloat16* out, float* out32, int ldo, int o_off, int relu,
            const __nv_bfloat16* mask, int ldm, int m_off, int mask_lo);
  void ensure(int nx, int ny, int B, bool grads);
  void release_acts();
  void conv_fwd(Ctx& c, int l, int lev, int B, const __nv_bfloat16* in, int ldi, int i_off, __nv_bfloat16* out,
                int ldo, int o_off, int relu, float* out32);
  void conv_bwd(Ctx& c, int l, int lev, int B, const __nv_bfloat16* in, int ldi, int i_off,
                const __nv_bfloat16* dout, int ldd, int d_off, __nv_bfloat16* din, int ldn, int n_off,
                const __nv_bfloat16* mask, int ldm, int mask_lo);

  long long woff_[kLayers] = {};
  long long wtotal_ = 0;
  float* w32_ = nullptr;
  __nv_bfloat16* wbf_ = nullptr;
  __nv_bfloat16* wt_ = nullptr;  // flipped weights of the data-gradient convolutions
  float* g32_ = nullptr;
  float* m_ = nullptr;
  float* v_ = nullptr;
  long long step_ = 0;
  // activations (forward) and their gradients, bf16
  int nx_ = 0, ny_ = 0, B_ = 0;
  bool grads_ = false;
  int gx_[4] = {}, gy_[4] = {};
  __nv_bfloat16* act_[11] = {};
  __nv_bfloat16* grd_[11] = {};
  float* y32_ = nullptr;
  float* x4_ = nullptr;
  long long x4cap_ = 0;
  float* scale_ = nullptr;
  int scalecap_ = 0;
  double* loss_ = nullptr;
  // training staging
  float* bx_ = nullptr;
  float* bt_ = nullptr;
  int* perm_ = nullptr;
  long long bcap_ = 0;
  int conv_path_ = 2;  // per layer the faster path (here: the tensor cores)
  int* tc_err_ = nullptr;
  __nv_bfloat16* wimg_ = nullptr;  // tensor-core weight images of the forward layers (at woff_)
  bool use_tc(int Cin, int Cout) const;
  void refresh_images(Ctx& c);
};

// 3x3 (2D, 9 taps) or 3x3x3 (3D, 27 taps) convolution on the 5th-generation
// tensor cores (hz_conv_tc.cu): Cin a multiple of 16 in [16, 256], Cout (the MMA
// width) a multiple of 16 in [16, 256] of which the first Cst (a multiple of 8)
// are stored; layouts as for the warp-level kernels except the weights, which
// come as the image that conv_tc_weight_image writes; *err is set when a wait
// timed out.
struct ConvTc {
  int nx, ny, nz, B;  // nz = 1: a 2D grid
  bool taps3d;        // 27 taps (needs nz > 1) or 9
  int Cin;
  const __nv_bfloat16* in;
  int ldi, i_off;
  int Cout, Cst;
  const __nv_bfloat16* wimg;
  __nv_bfloat16* out;
  float* out32;
  int ldo, o_off, relu;
  const __nv_bfloat16* mask;
  int ldm, m_off, mask_lo;
};
bool conv_tc_supported(int taps, int Cin, int Cout);
void conv_tc_launch(Ctx& ctx, const char* name, const ConvTc& a, int* err);
// Weight gradient on the 5th-generation tensor cores (hz_conv_tc.cu):
// dw [Cout][taps][Cin] (FP32) += sum over the nodes of dout[n][co] * in[n + off_t][ci],
// taps = 27 when nz > 1 else 9; Cin a multiple of 16 in [16, 128], Cout a
// multiple of 8 in [8, 128]; nodes = B * nx * ny * nz rows; *err is set when a
// wait timed out.
struct WgradTc {
  int nx, ny, nz;
  long long nodes;
  int Cin;
  const __nv_bfloat16* in;
  int ldi;
  int Cout;
  const __nv_bfloat16* dout;
  int ldd, d_off;
  float* dw;
};
bool wgrad_tc_supported(int taps, int Cin, int Cout);
void wgrad_tc_launch(Ctx& ctx, const char* name, const WgradTc& a, int* err);
// Weight image of a convolution with taps taps, Cin inputs and Cout outputs
// (taps * Cin * Cout BF16 values): flip = 0 from w [wcout][taps][Cin] (outputs
// >= wcout are zero); flip = 1 the data-gradient weights of a layer
// w [wcout][taps][wcin] (wcin = Cout; inputs >= wcout are zero).
void conv_tc_weight_image(Ctx& ctx, const char* name, int taps, int Cin, int Cout, const __nv_bfloat16* w, int flip,
                          int wcin, int wcout, __nv_bfloat16* img);

// 3D convolutional encoder-decoder of the same kind (three grid levels, 8-16-32
// channels, 3x3x3 convolutions; the layers and their order are in hz_learn3d.cu):
//   input  x [B][N][4] FP32 and output y [B][N][8] FP32 as for the 2D network,
//   N = nx * ny * nz, axis 1 fastest; n - 1 divisible by 4 on every axis.
// Weights exchanged with the host: layer after layer, each [cout][27][cin] with
// tap t = 9 (dz + 1) + 3 (dy + 1) + (dx + 1).
class CoarseNet3 {
 public:
  static constexpr int kLayers = 6;
  explicit CoarseNet3(unsigned seed);
  ~CoarseNet3();
  CoarseNet3(const CoarseNet3&) = delete;
  CoarseNet3& operator=(const CoarseNet3&) = delete;

  static long long num_params();
  static bool supports(long long nx, long long ny, long long nz);
  static void layer_shape(int l, int* cin, int* cout);

  void get_weights(float* host) const;
  void set_weights(const float* host);
  void get_grad(float* host) const;
  void save(const char* path) const;
  void load(const char* path);
  static int file_info(const char* path, long long* nparams, long long* step);

  void forward(Ctx& c, const float* x4, int nx, int ny, int nz, int B, bool train = false);
  const float* output() const { return y32_; }
  float* input_staging(int nx, int ny, int nz, int B);
  float* scale_staging(int B);
  double backward(Ctx& c, const float* t, int nx, int ny, int nz, int B);
  void adam(Ctx& c, double lr);
  void train(Ctx& c, const float* x, const float* t, int nx, int ny, int nz, long long nsamples, int batch,
             int epochs, double lr, unsigned seed, double* loss_hist);

  Ctx ctx;

  // convolution kernels, as for the 2D network: 0 = warp-level MMA; 1 =
  // 5th-generation tensor cores for every layer; 2 (the default) = per layer
  // the faster of the two, by the waste of the tensor-core tiles on the
  // layer's grid (tc_waste in hz_learn3d.cu)
  void set_conv_path(int path);
  int conv_path() const { return conv_path_; }
  bool tc_failed();

 private:
  void ensure(int nx, int ny, int nz, int B, bool grads);
  void release_acts();
  bool use_tc(int Cin, int Cout, int lev) const;
  void refresh_images(Ctx& c);
  void conv_fwd(Ctx& c, int l, int B, const __nv_bfloat16* in, int ldi, int i_off, __nv_bfloat16* out, int ldo,
                int o_off, int relu, float* out32);
  void conv_bwd(Ctx& c, int l, int B, const __nv_bfloat16* in, int ldi, const __nv_bfloat16* dout, int ldd,
                int d_off, __nv_bfloat16* din, int ldn, int n_off, const __nv_bfloat16* mask, int ldm, int mask_lo);

  long long woff_[kLayers] = {};
  long long wtotal_ = 0;
  float* w32_ = nullptr;
  __nv_bfloat16* wbf_ = nullptr;
  __nv_bfloat16* wt_ = nullptr;
  float* g32_ = nullptr;
  float* m_ = nullptr;
  float* v_ = nullptr;
  long long step_ = 0;
  int g_[3][3] = {};  // node counts (x, y, z) of the network's three grids
  int B_ = 0;
  bool grads_ = false;
  __nv_bfloat16* act_[8] = {};
  __nv_bfloat16* grd_[8] = {};
  float* y32_ = nullptr;
  float* x4_ = nullptr;
  long long x4cap_ = 0;
  float* scale_ = nullptr;
  int scalecap_ = 0;
  double* loss_ = nullptr;
  float* bx_ = nullptr;
  float* bt_ = nullptr;
  int* perm_ = nullptr;
  long long bcap_ = 0;
  int conv_path_ = 2;  // per layer the faster path
  int* tc_err_ = nullptr;
  __nv_bfloat16* wimg_ = nullptr;  // tensor-core weight images of the forward layers (at imgoff_)
  long long imgoff_[kLayers] = {};
  long long imgtotal_ = 0;
};

// Kernels the 2D and 3D networks share (hz_learn.cu): input assembly into
// 16-channel rows, the loss and its gradient, Adam, FP32 -> BF16, and the
// mini-batch gather of training pairs.
__global__ void k_pack_in(long long BN, const float4* __restrict__ x4, __nv_bfloat16* __restrict__ x16);
__global__ void __launch_bounds__(256) k_loss(int N, int B, const float* __restrict__ y, const float* __restrict__ t,
                                              __nv_bfloat16* __restrict__ dy, double* __restrict__ loss);
__global__ void k_adam(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2, float eps,
                       float c1, float c2);
__global__ void k_f2bf(long long n, const float* __restrict__ a, __nv_bfloat16* __restrict__ b);
__global__ void k_gather_pairs(int B, long long N, const int* __restrict__ perm, const float4* __restrict__ x,
                               const float2* __restrict__ t, float4* __restrict__ bx, float2* __restrict__ bt);

// Column RMS s_k of the active columns of b (one level, ld-strided), then the
// network input x[k][p] = (b/s, feat[p]) (conj: the adjoint solve feeds conj(b)).
template <typename T>
void launch_net_pack(Ctx& ctx, long long N, const cplx<T>* b, long long ld, const int* cols, int nc,
                     const float2* feat, int conj, float* scale, float* x4);
// out[cols[k]] = s_k h2 (y0 + i y1) (conj: conjugated)
template <typename T>
void launch_net_unpack(Ctx& ctx, long long N, const float* y, const float* scale, double h2, int conj, cplx<T>* out,
                       long long ld, const int* cols, int nc);
// Training pairs from compact FP64 columns r, e (k = 0..nc): x as in launch_net_pack
// and t = e / (h2 s_k); scale receives s_k.
void launch_pair_pack(Ctx& ctx, long long N, const double2* r, const double2* e, int nc, const float2* feat,
                      double h2, float* scale, float* x4, float* t2);
// Compact-column helpers (FP64): gather active columns, x += e, and per-column
// sums |a - b|^2, |a|^2 and |b|^2 into out[3k], out[3k+1], out[3k+2].
void launch_gather_cols(Ctx& ctx, long long N, const double2* src, long long ld, const int* cols, int nc,
                        double2* dst);
void launch_axpy_compact(Ctx& ctx, long long N, int nc, const double2* e, double2* x);
void launch_diff_norms(Ctx& ctx, long long N, int nc, const double2* a, const double2* b, double* out);

}  // namespace hz
