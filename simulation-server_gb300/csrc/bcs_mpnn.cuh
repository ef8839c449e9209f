// bcs_mpnn.cuh — the learned sub-step network: layout of its parameters and
// the kernels' entry points.
//
// A message-passing network over one blood cell's spring graph (hidden 128):
//     h0 = silu(f W_in + b_in)                       f: 16 node features
//     layer l: B   = silu(h W_b + b_b)                node messages
//              M_i = mean over the springs of i of B_j + ebar_i W_e + b_e
//              h   = h + silu(h W_u + M W_v + b_u)
//     y = h W_out + b_out                            y: 9 outputs per node
// ebar_i is the mean of node i's 8 edge features.  Weights are bfloat16 (an
// FP32 master copy is what the optimiser updates); the hidden x hidden
// products run on the tensor cores with FP32 accumulation, everything else
// in FP32.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

namespace bcs {

constexpr int kHidden = 128;
constexpr int kFeatIn = 16;
constexpr int kEdgeIn = 8;
constexpr int kOut = 9;
constexpr int kMaxLayers = 4;

// Offsets (in floats) of each parameter tensor in the flat parameter vector.
struct MpnnLayout {
    int layers = 3;
    long long w_in, b_in, w_out, b_out;
    long long wb[kMaxLayers], bb[kMaxLayers], we[kMaxLayers], be[kMaxLayers];
    long long wu[kMaxLayers], wv[kMaxLayers], bu[kMaxLayers];
    long long total = 0;
};

inline MpnnLayout mpnn_layout(int layers) {
    MpnnLayout L;
    L.layers = layers;
    long long o = 0;
    auto take = [&](long long n) { long long r = o; o += n; return r; };
    L.w_in = take((long long)kFeatIn * kHidden);
    L.b_in = take(kHidden);
    for (int l = 0; l < layers; ++l) {
        L.wb[l] = take((long long)kHidden * kHidden);
        L.bb[l] = take(kHidden);
        L.we[l] = take((long long)kEdgeIn * kHidden);
        L.be[l] = take(kHidden);
        L.wu[l] = take((long long)kHidden * kHidden);
        L.wv[l] = take((long long)kHidden * kHidden);
        L.bu[l] = take(kHidden);
    }
    L.w_out = take((long long)kHidden * kOut);
    L.b_out = take(kOut);
    L.total = o;
    return L;
}

// The graph of a batch: `cells` copies of one cell's CSR graph (pic nodes).
struct MpnnGraph {
    int cells, pic;
    const int* adj_off;    // pic + 1 offsets
    const int* adj_nbr;    // neighbour within the cell
    const float* adj_len;  // rest length of the spring
};

// ---- kernels (bcs_mpnn.cu); every matrix is row-major, rows = nodes ------
// Y = epi(X1 W1 + X2 W2 + bias) for hidden x hidden W, each passed as its
// transposed bf16 copy W^T ([out][in]); X2/W2 may be null.  silu applies
// silu; Zout (optional) receives the pre-activation; accumulate adds to Y.
void mpnn_gemm(const float* X1, const __nv_bfloat16* W1t, const float* X2, const __nv_bfloat16* W2t,
               const float* bias, float* Y, float* Zout, int rows, bool silu, bool accumulate, cudaStream_t s);
// Which tensor-core instructions the products use: 0 = tcgen05 (TMEM
// accumulators, the default), 1 = mma.sync.  The error word counts tcgen05
// waits that expired.
void mpnn_set_gemm_path(int path);
bool mpnn_set_wait_probe(int polls);
int mpnn_gemm_path();
unsigned* mpnn_gemm_error_word();
// dX (+)= dY W^T for hidden x hidden W.
void mpnn_gemm_t(const float* dY, const __nv_bfloat16* W, float* dX, int rows, bool accumulate, cudaStream_t s);
// dW += X^T dY (FP32 atomics into dW [hidden][hidden]), both operands rounded to bf16.
void mpnn_wgrad(const float* X, const float* dY, float* dW, int rows, cudaStream_t s);

// The network with its optimiser state and activation buffers for batches
// of up to `max_cells` cells of one graph.  All work is enqueued on `stream`.
class MpnnNet {
public:
    MpnnNet() = default;
    ~MpnnNet();
    MpnnNet(const MpnnNet&) = delete;
    MpnnNet& operator=(const MpnnNet&) = delete;
    // Host CSR graph of one cell (pic nodes); returns a cudaError_t value.
    int init(int layers, int pic, const int* adj_off, const int* adj_nbr, const float* adj_len, int max_cells,
             unsigned long long seed, cudaStream_t stream);
    // f [cells*pic][16], E [cells*edges][8] (normalised) -> Y [cells*pic][9];
    // keep = false reuses one set of layer buffers (inference).
    void forward(const float* f, const float* E, int cells, bool keep);
    // loss of the last forward (keep = true) against T, gradients into grad().
    void backward(const float* T, int cells);
    void adam(float lr);
    void refresh_bf16();
    void set_huber(float delta) { huber_ = delta; }
    float* params() { return p_; }
    float* grad() { return g_; }
    float* output() { return y_; }
    float* loss_dev() { return loss_; }
    float* input_buf() { return f_; }
    float* edge_buf() { return e_; }
    float* target_buf() { return t_; }
    long long param_count() const { return L_.total; }
    int edges() const { return edges_; }
    int pic() const { return pic_; }
    int max_cells() const { return max_cells_; }
    int layers() const { return L_.layers; }
    const int* dev_adj_off() const { return adj_off_; }
    const int* dev_adj_nbr() const { return adj_nbr_; }
    const float* dev_adj_len() const { return adj_len_; }
    const __nv_bfloat16* weights_bf16() const { return pb_; }
    const __nv_bfloat16* weights_bf16_t() const { return pbt_; }
    const MpnnLayout& layout() const { return L_; }
    size_t bytes() const { return bytes_; }

private:
    float* alloc(size_t n);
    MpnnLayout L_;
    cudaStream_t st_ = nullptr;
    int pic_ = 0, edges_ = 0, max_cells_ = 0;
    int *adj_off_ = nullptr, *adj_nbr_ = nullptr, *edge_base_ = nullptr;
    float* adj_len_ = nullptr;
    float *p_ = nullptr, *g_ = nullptr, *m_ = nullptr, *v_ = nullptr;
    __nv_bfloat16 *pb_ = nullptr, *pbt_ = nullptr;
    long long* sq_ = nullptr;
    int nsq_ = 0, t_adam_ = 0;
    float huber_ = 0.f;
    float *f_ = nullptr, *e_ = nullptr, *t_ = nullptr, *y_ = nullptr, *dy_ = nullptr, *loss_ = nullptr;
    const float *last_f_ = nullptr, *last_e_ = nullptr;   // inputs of the last forward
    float *z0_ = nullptr, *dh_ = nullptr, *db_ = nullptr, *dm_ = nullptr, *dz_ = nullptr;
    float *h_[kMaxLayers + 1] = {}, *zb_[kMaxLayers] = {}, *b_[kMaxLayers] = {}, *mm_[kMaxLayers] = {},
          *zu_[kMaxLayers] = {};
    std::vector<void*> allocs_;
    size_t bytes_ = 0;
};

}  // namespace bcs
