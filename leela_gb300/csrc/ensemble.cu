// ensemble.cu -- the 8-symmetry ensemble (AVERAGE_ALL) on the device.
//
// Reference: Network::get_scored_moves(AVERAGE_ALL) evaluates the policy net
// on the position under each of the 8 dihedral symmetries, un-rotates each
// result and averages them (Network.cpp:642-654); get_value(AVERAGE_ALL)
// averages the 8 values (Network.cpp:606-615).  Here the 8 rotated copies of
// every position are one batch: a kernel writes them (rotation tables of
// Network.cpp:1341-1379 in constant memory), the nets run once at batch 8B,
// and a second kernel un-rotates and averages.
#include "lg_kernels.h"

namespace lg {

__constant__ short c_rot[8][kPoints];     // rotate_nn_idx(i, s)
__constant__ short c_rev_rot[8][kPoints]; // rev_rotate_nn_idx(i, s)

static int rotate_idx(int v, int s) {
    int x = v % kBoard, y = v / kBoard;
    if (s >= 4) {
        int t = x;
        x = y;
        y = t;
        s -= 4;
    }
    int nx = (s & 2) ? kBoard - 1 - x : x;
    int ny = (s & 1) ? kBoard - 1 - y : y;
    return ny * kBoard + nx;
}

int ensemble_init_tables() {
    static const int inv[8] = {0, 1, 2, 3, 4, 6, 5, 7};
    short rot[8][kPoints], rev[8][kPoints];
    for (int s = 0; s < 8; ++s)
        for (int i = 0; i < kPoints; ++i) {
            rot[s][i] = (short)rotate_idx(i, s);
            rev[s][i] = (short)rotate_idx(i, inv[s]);
        }
    if (cudaMemcpyToSymbol(c_rot, rot, sizeof rot) != cudaSuccess ||
        cudaMemcpyToSymbol(c_rev_rot, rev, sizeof rev) != cudaSuccess) {
        lg_set_error("could not upload the rotation tables");
        return LG_ERR_CUDA;
    }
    return LG_OK;
}

// out[b*8 + s][c][i] = in[b][c][rotate(i, s)]
__global__ void rotate8_kernel(const uint8_t *__restrict__ in, int B, int C, uint8_t *__restrict__ out) {
    const size_t total = (size_t)B * 8 * C * kPoints;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(k % kPoints);
        const size_t rest = k / kPoints;
        const int c = (int)(rest % C);
        const size_t bs = rest / C;
        const int s = (int)(bs % 8);
        const size_t b = bs / 8;
        out[k] = in[(b * C + c) * kPoints + c_rot[s][i]];
    }
}

// avg[b][i] = 1/8 sum_s probs[b*8 + s][rev_rotate(i, s)]  (board order)
__global__ void unrotate_avg8_kernel(const float *__restrict__ probs, int B, float *__restrict__ avg) {
    const int b = blockIdx.x, i = threadIdx.x;
    if (b >= B || i >= kPoints) return;
    float s = 0.0f;
#pragma unroll
    for (int r = 0; r < 8; ++r) s += probs[((size_t)b * 8 + r) * kPoints + c_rev_rot[r][i]];
    avg[(size_t)b * kPoints + i] = s / 8.0f;
}

__global__ void avg8_kernel(const float *__restrict__ v, int B, float *__restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float s = 0.0f;
#pragma unroll
    for (int r = 0; r < 8; ++r) s += v[(size_t)b * 8 + r];
    out[b] = s / 8.0f;
}

void launch_rotate8(const uint8_t *in, int B, int C, uint8_t *out, cudaStream_t s) {
    size_t total = (size_t)B * 8 * C * kPoints;
    int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
    rotate8_kernel<<<blocks, 256, 0, s>>>(in, B, C, out);
}
void launch_unrotate_avg8(const float *probs, int B, float *avg, cudaStream_t s) {
    unrotate_avg8_kernel<<<B, 384, 0, s>>>(probs, B, avg);
}
void launch_avg8(const float *v, int B, float *out, cudaStream_t s) {
    avg8_kernel<<<(B + 127) / 128, 128, 0, s>>>(v, B, out);
}

}  // namespace lg
