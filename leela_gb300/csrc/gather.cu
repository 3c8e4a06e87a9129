// gather.cu -- the input planes on the GPU, from a compact board encoding.
//
// Reference: Network::gather_features_policy / gather_features_value
// (Network.cpp:883-1046, 1048-1201) build 32 planes per position on the host
// from FastBoard queries; planes 0..23 of both sets -- the ones the
// benchmark nets read -- need only stone colours, the liberty count of each
// string (FastBoard::count_rliberties, FastBoard.cpp:2482-2508) and, for
// each empty point, the liberties of the string a stone of either colour
// would form there after its captures, 0 for a suicide
// (FastBoard::after_liberties, FastBoard.cpp:2511-2528).  Planes 24..31
// (ladders, ko, move history, komi, third line) are not produced here.
//
// One CTA per board, one thread per point.  Strings are labelled by
// propagating the minimum point index over same-coloured neighbours; every
// string root owns two 361-bit sets in shared memory (its stones, and the
// points adjacent to any of its stones), so that
//   liberties(string)            = |adj & empty|
//   after-move liberties(p, c)   = |(nbrs(p) | adj of c's strings next to p)
//                                   & ((empty | stones of captured strings) - {p})|
// where the captured strings are the opponent strings next to p with one
// liberty.
//
// Input: squares [B][361] (0 black, 1 white, 2 empty; point y*19+x), to_move
// [B] (0 black, 1 white).  Output: planes [B][nplanes][361] bytes (0/1).
#include "lg_kernels.h"

namespace lg {

constexpr int kWords = (kPoints + 31) / 32;  // 12

__device__ __forceinline__ int nbr(int p, int k) {
    const int x = p % kBoard, y = p / kBoard;
    switch (k) {
    case 0: return x > 0 ? p - 1 : -1;
    case 1: return x < kBoard - 1 ? p + 1 : -1;
    case 2: return y > 0 ? p - kBoard : -1;
    default: return y < kBoard - 1 ? p + kBoard : -1;
    }
}

template <int WHICH>  // 0 = policy planes, 1 = value planes
__global__ void __launch_bounds__(384) gather_kernel(const int8_t *__restrict__ squares,
                                                     const int8_t *__restrict__ to_move, int B,
                                                     int nplanes, uint8_t *__restrict__ planes) {
    __shared__ int8_t sq[kPoints];
    __shared__ short lab[kPoints];
    __shared__ uint32_t stones[kPoints][kWords];
    __shared__ uint32_t adj[kPoints][kWords];
    __shared__ uint32_t empty[kWords];
    __shared__ short libs[kPoints];
    const int b = blockIdx.x;
    if (b >= B) return;
    const int p = threadIdx.x;
    const bool on = p < kPoints;
    const int tomove = to_move[b];
    int8_t c = 2;
    if (on) {
        c = squares[(size_t)b * kPoints + p];
        sq[p] = c;
        lab[p] = (c == 2) ? -1 : (short)p;
        for (int w = 0; w < kWords; ++w) {
            stones[p][w] = 0;
            adj[p][w] = 0;
        }
    }
    if (p < kWords) empty[p] = 0;
    __syncthreads();
    // string labels: minimum point index of the string
    for (int it = 0; it < 2 * kPoints; ++it) {
        int changed = 0;
        if (on && c != 2) {
            int m = lab[p];
            for (int k = 0; k < 4; ++k) {
                const int q = nbr(p, k);
                if (q >= 0 && sq[q] == c) m = min(m, (int)lab[q]);
            }
            m = min(m, (int)lab[m]);  // jump towards the root
            if (m < lab[p]) {
                lab[p] = (short)m;
                changed = 1;
            }
        }
        if (!__syncthreads_or(changed)) break;
    }
    if (on) {
        if (c == 2) {
            atomicOr(&empty[p >> 5], 1u << (p & 31));
        } else {
            const int r = lab[p];
            atomicOr(&stones[r][p >> 5], 1u << (p & 31));
            for (int k = 0; k < 4; ++k) {
                const int q = nbr(p, k);
                if (q >= 0) atomicOr(&adj[r][q >> 5], 1u << (q & 31));
            }
        }
    }
    __syncthreads();
    if (on && c != 2 && lab[p] == p) {
        int n = 0;
        for (int w = 0; w < kWords; ++w) n += __popc(adj[p][w] & empty[w]);
        libs[p] = (short)n;
    }
    __syncthreads();
    if (!on) return;
    uint32_t bits = 0;  // bit i = plane i at this point
    if (c != 2) {
        const bool mine = c == tomove;
        bits |= mine ? 2u : 4u;
        const int l = libs[lab[p]];
        if (WHICH == 0) {  // policy: 1, 2, 3, 4, 5+ ; own at 3.., opponent at 8..
            if (l >= 1) bits |= 1u << ((mine ? 3 : 8) + (l >= 5 ? 4 : l - 1));
        } else {           // value: 1, 2, 3, 4, 5, 6+ ; own at 3.., opponent at 9..
            if (l >= 1) bits |= 1u << ((mine ? 3 : 9) + (l >= 6 ? 5 : l - 1));
        }
    } else {
        bits |= 1u;
        int nb[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) nb[k] = nbr(p, k);
        // liberties after a stone of colour col is played here
        int after[2];
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int col = side == 0 ? tomove : !tomove;
            // the strings next to p: joined (own colour) or captured
            // (opponent's with one liberty, which is p); -1 = none
            int join[4], capt[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                join[k] = -1;
                capt[k] = -1;
                const int q = nb[k];
                if (q < 0) continue;
                const int cq = sq[q];
                if (cq == col) join[k] = lab[q];
                else if (cq != 2 && libs[lab[q]] == 1) capt[k] = lab[q];
            }
            int n = 0;
            for (int w = 0; w < kWords; ++w) {
                uint32_t u = 0, e = empty[w];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int q = nb[k];
                    if (q >= 0 && (q >> 5) == w) u |= 1u << (q & 31);
                    if (join[k] >= 0) u |= adj[join[k]][w];
                    if (capt[k] >= 0) e |= stones[capt[k]][w];
                }
                if (w == (p >> 5)) e &= ~(1u << (p & 31));
                n += __popc(u & e);
            }
            after[side] = n;
        }
        const int al = after[0], at = after[1];
        if (WHICH == 0) {  // after 1..6+ at 13..18, opponent 1..5 at 19..23
            if (al >= 1) bits |= 1u << (13 + (al >= 6 ? 5 : al - 1));
            if (at >= 1 && at <= 5) bits |= 1u << (19 + at - 1);
        } else {           // after 1..6+ at 15..20, opponent 1..3 at 21..23
            if (al >= 1) bits |= 1u << (15 + (al >= 6 ? 5 : al - 1));
            if (at >= 1 && at <= 3) bits |= 1u << (21 + at - 1);
        }
    }
    uint8_t *dst = planes + (size_t)b * nplanes * kPoints + p;
    for (int i = 0; i < nplanes; ++i) dst[(size_t)i * kPoints] = (uint8_t)((bits >> i) & 1u);
}

int launch_gather(const int8_t *squares, const int8_t *to_move, int B, int which, int nplanes,
                  uint8_t *planes, cudaStream_t s) {
    if (B < 0 || nplanes < 1 || nplanes > kGatherPlanes || (which != 0 && which != 1)) {
        lg_set_error("gather: planes 0..23 of the policy (0) or value (1) set only");
        return LG_ERR_ARG;
    }
    if (B == 0) return LG_OK;
    if (which == 0)
        gather_kernel<0><<<B, 384, 0, s>>>(squares, to_move, B, nplanes, planes);
    else
        gather_kernel<1><<<B, 384, 0, s>>>(squares, to_move, B, nplanes, planes);
    return LG_OK;
}

}  // namespace lg

extern "C" int lg_gather_device(const int8_t *squares, const int8_t *to_move, int B, int which, int nplanes,
                                uint8_t *planes, void *stream) {
    if ((!squares || !to_move || !planes) && B > 0) {
        lg_set_error("lg_gather_device: bad arguments");
        return LG_ERR_ARG;
    }
    int rc = lg::launch_gather(squares, to_move, B, which, nplanes, planes, (cudaStream_t)stream);
    if (rc) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        lg_set_error("lg_gather_device: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}
