// ose_learn.h - the learned-boundary corrector (ose_learn.cu): geometry,
// device buffers and launch helpers shared with the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/ose3d.h"

namespace ose {
namespace learn {

constexpr int kLayers = 4;
extern const int kCin[kLayers];
extern const int kCout[kLayers];

// Padded grid, shell width and sponge widths (x-, x+, y-, y+, z-, z+).
struct NetGeom {
    int nx, ny, nz;
    int shell;
    int sp[6];
};

// One network instance on one grid: parameters and every work buffer
// (device pointers; dense over the padded grid, channels last).
struct Net {
    NetGeom g;
    int* tiles;            // 8^3 tiles meeting the shell, packed i | j << 10 | k << 20
    int ntiles;
    long long ncells;      // shell cells
    long long nwrite;      // write cells (shell outside the sponge)
    float* params;         // param_count() floats
    float* grads;
    float* m;
    float* v;
    float* wt[kLayers];    // data-gradient weights of layers 1..3
    float* F;              // [cell][8] input features
    float* A[3];           // [cell][32] hidden activations
    float* O;              // [cell][2] output
    float* G4;             // [cell][2] output gradient
    float* GA[3];          // [cell][32] gradients of the hidden activations
    float* scal;           // [0] sum of squares over the shell, [1] its RMS, [2] 1/RMS
    float* sloc;           // [cell] local scale s(x)
    float* stmp;           // [cell] box-sum scratch
    float* loss;           // [0] accumulated loss
};

// Tensor-core inference (ose_learn_tc.cu): BF16 weights per layer in the
// kernel's shared-memory layout, biases padded to the layer's N, BF16
// ping-pong activations [cell][32], and the columns of 8 x 16 output planes
// (two ints each: x tile | y tile << 10, z0 | planes << 16).
struct TcNet {
    int* tiles;
    int ntiles;
    uint8_t* w[kLayers];
    float* b[kLayers];
    uint16_t* act[2];
    int* err;              // device error word (a wait that ran out of time)
};

size_t param_offset(int layer);
size_t param_count();
void shell_tiles(const NetGeom& g, std::vector<int>& tiles, long long* ncells, long long* nwrite);
cudaError_t configure();
// Forward pass on state W (float2 P + iQ, [z][y][x]) and velocity vel.  With
// apply, adds the correction to state_out (may equal W); else writes n.O.
// scale = false: n.sloc / n.scal already hold this state's local scale
cudaError_t forward(cudaStream_t s, const Net& n, const float2* W, const float* vel, bool apply, float2* state_out,
                    bool scale = true);
// Forward + backward of one sample; gradients add into n.grads, loss into n.loss.
cudaError_t train_sample(cudaStream_t s, const Net& n, const float2* W, const float* vel, const float2* tgt);
// One Adam update with gradients scaled by gscale; clears the gradients.
cudaError_t adam(cudaStream_t s, const Net& n, float lr, float b1, float b2, float eps, int step, float gscale);

// Shell RMS -> n.scal[1], 1/RMS -> n.scal[2]; local scale s(x) -> n.sloc.
cudaError_t shell_scale(cudaStream_t s, const Net& n, const float2* W);
void tc_layer_weights(const float* w, int cin, int cout, int cin_pad, int npad, std::vector<uint8_t>& out);
void tc_tiles(const NetGeom& g, std::vector<int>& tiles);
cudaError_t configure_tc();
// state += s * corrector(state) at the write cells, on the tensor cores.
cudaError_t forward_tc(cudaStream_t s, const Net& n, const TcNet& tc, float2* W, const float* vel,
                       bool scale = true);

// Corrector objects (the C ABI's ose_corrector) for the modeler's own use.
ose_corrector* new_corrector();
void delete_corrector(ose_corrector* c);
cudaError_t create_net(ose_corrector* c, const NetGeom& g, bool training, bool fp32_forward);
const Net& net_of(const ose_corrector* c);
// Tensor-core buffers for inference from FP32 host parameters; err = the
// device error word the kernels report to.
cudaError_t create_tc(ose_corrector* c, const float* params_host, int* err);
const TcNet* tc_of(const ose_corrector* c);

}  // namespace learn
}  // namespace ose
