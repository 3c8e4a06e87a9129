// gather.cu -- the input planes on the GPU, from a compact board encoding.
//
// Reference: Network::gather_features_policy / gather_features_value
// (Network.cpp:883-1046, 1048-1201) build 32 planes per position on the host
// from FastBoard queries: stone colours, the liberty count of each string
// (FastBoard::count_rliberties, FastBoard.cpp:2482-2508), for each empty
// point the liberties of the string a stone of either colour would form
// there after its captures, 0 for a suicide (FastBoard::after_liberties,
// FastBoard.cpp:2511-2528), the ladder reader's two planes (ladder.cuh), the
// ko point, the last two moves, white's komi and the third line.  Planes
// 0..23 -- the benchmark nets' inputs -- need only the board.
//
// One CTA per board, one thread per point.  Strings are labelled with their
// minimum point index by a union-find over same-coloured neighbours; every
// string root owns two 361-bit sets in shared memory (its stones, and the
// points adjacent to any of its stones), so that
//   liberties(string)            = |adj & empty|
//   after-move liberties(p, c)   = |(nbrs(p) | adj of c's strings next to p)
//                                   & ((empty | stones of captured strings) - {p})|
// where the captured strings are the opponent strings next to p with one
// liberty.  Most empty points (no capture, at most one string joined) need
// no set: the count is then the empty neighbours, or the joined string's
// liberties less p plus the empty neighbours outside its adjacency.
//
// Planes 24..31: the ladder reader runs only where it can answer "yes" --
// an empty point with two empty neighbours next to an own string in atari
// (ladder), or next to an opponent string of two liberties (ladder win).
// The point threads list those candidates in shared memory; then each warp
// takes candidates from the list and reads the ladder on a row bitboard
// (ladder.cuh), all 32 lanes together.
//
// Input: squares [B][361] (0 black, 1 white, 2 empty; point y*19+x), to_move
// [B] (0 black, 1 white), and for planes 24..31 moves [B][4] (last move, the
// move before it, ko point: point indices, -1 none; white-has-komi flag).
// Output: planes [B][nplanes][361] bytes (0/1).
#include "lg_kernels.h"
#include "ladder.cuh"

namespace lg {
using namespace ptx;

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

// union-find over the points of one board (shared memory); par[x] <= x,
// and parents only decrease.  A path to the root strictly decreases, so it
// has at most x < kPoints steps: the loop bound is never what ends it.
__device__ __forceinline__ int find_root(const volatile int *par, int x) {
    for (int i = 0; i < kPoints && par[x] != x; ++i) x = par[x];
    return x;
}

// joins the trees of a and b: the larger root is linked under the smaller
// (atomicMin); if it stopped being a root meanwhile, the atomicMin has moved
// its link and the join goes on from the parent it had.  Every retry starts
// from two roots below the previous larger root (both roots are at most the
// parent found, which is below it), so there are fewer than kPoints
// rounds: the bound of 4 * kPoints is never what ends the loop.
__device__ void unite(int *par, int a, int b) {
    for (int i = 0; i < 4 * kPoints; ++i) {
        a = find_root(par, a);
        b = find_root(par, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicMin(&par[a], b);
        if (old == a) return;
        a = old;
    }
}

// WHICH: 0 = policy planes, 1 = value planes; EXTRA: planes 24..31 wanted
// (the ladder reader's code and shared lists stay out of the 24-plane
// kernel); L5: write the first layer's expanded input rows (l5, `halves` x 64
// 16-bit channels a row, 1.0 encoded as `one`: 0x3F80 for BF16, 0x3C00 for
// FP16) instead of the planes
template <int WHICH, bool EXTRA, bool L5>
__device__ __forceinline__ void gather_board(const int8_t *__restrict__ squares, const int8_t *__restrict__ to_move,
                                             const int32_t *__restrict__ moves, int B, int nplanes,
                                             uint8_t *__restrict__ planes, int halves, uint32_t one,
                                             uint4 *__restrict__ l5) {
    constexpr bool extra = EXTRA;
    constexpr int kCand = extra ? 2 * kPoints : 1;
    __shared__ uint32_t rowc[2][kBoard];  // row bitboard: bit x of rowc[c][y] = stone of colour c at (y, x)
    __shared__ short cand[kCand];         // ladder candidates: point | kind << 9 (0 ladder, 1 ladder win)
    __shared__ uint8_t lad_yes[extra ? kPoints : 1], win_yes[extra ? kPoints : 1];
    __shared__ int ncand;
    __shared__ int8_t sq[kPoints];
    __shared__ short lab[kPoints];
    __shared__ __align__(16) uint32_t stones[kPoints][kWords];
    __shared__ __align__(16) uint32_t adj[kPoints][kWords];
    __shared__ uint32_t empty[kWords];
    __shared__ short libs[kPoints];
    __shared__ int par[kPoints];                     // union-find parents
    __shared__ uint32_t pbits[L5 ? kPoints : 1];     // the planes of each point, for the L5 rows
    __shared__ uint8_t adj_lo[kPoints], adj_hi[kPoints];  // words of a root's adjacency set
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
        uint4 *zs = reinterpret_cast<uint4 *>(stones[p]), *za = reinterpret_cast<uint4 *>(adj[p]);
#pragma unroll
        for (int w = 0; w < kWords / 4; ++w) {
            zs[w] = make_uint4(0u, 0u, 0u, 0u);
            za[w] = make_uint4(0u, 0u, 0u, 0u);
        }
        if (extra) {
            lad_yes[p] = 0;
            win_yes[p] = 0;
        }
    }
    if (p < kWords) empty[p] = 0;
    if (extra && p < 2 * kBoard) rowc[p / kBoard][p % kBoard] = 0;
    if (extra && p == 0) ncand = 0;
    __syncthreads();
    // string labels: the minimum point index of the string, by union-find:
    // every stone links to its left and upper neighbours of its colour (the
    // larger root under the smaller), then follows its parents to the root
    if (on) par[p] = p;
    __syncthreads();
    if (on && c != 2) {
        if (p % kBoard > 0 && sq[p - 1] == c) unite(par, p, p - 1);
        if (p >= kBoard && sq[p - kBoard] == c) unite(par, p, p - kBoard);
    }
    __syncthreads();
    if (on && c != 2) lab[p] = (short)find_root(par, p);
    if (on) {
        if (c == 2) {
            atomicOr(&empty[p >> 5], 1u << (p & 31));
        } else {
            if (extra && (c == 0 || c == 1)) atomicOr(&rowc[c][p / kBoard], 1u << (p % kBoard));
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
        int n = 0, lo = kWords - 1, hi = 0;
        for (int w = 0; w < kWords; ++w) {
            const uint32_t a = adj[p][w];
            n += __popc(a & empty[w]);
            if (a) {
                lo = min(lo, w);
                hi = w;
            }
        }
        libs[p] = (short)n;
        adj_lo[p] = (uint8_t)lo;
        adj_hi[p] = (uint8_t)hi;
    }
    __syncthreads();
    uint32_t bits = 0;  // bit i = plane i at this point
    // policy: own libs 1,2,3,4,5+ at 3..7, opponent's at 8..12, after-move
    // 1..5,6+ at 13..18, opponent's after-move 1..5,6+ at 19..24, ladder 25,
    // ladder win 26, ko 27, last move 28, the move before 29, white's komi 30,
    // third line 31.  value: libs 1..5,6+ at 3..8 / 9..14, after-move 1..5,6+
    // at 15..20 / 21..26, ladder 27, ladder win 28, komi 29, third line 30,
    // ko 31.
    constexpr int kLibCap = WHICH == 0 ? 5 : 6, kOppLib0 = WHICH == 0 ? 8 : 9;
    constexpr int kAfter0 = WHICH == 0 ? 13 : 15, kOAfter0 = WHICH == 0 ? 19 : 21;
    constexpr int kLadder = WHICH == 0 ? 25 : 27, kWin = WHICH == 0 ? 26 : 28;
    constexpr int kKomi = WHICH == 0 ? 30 : 29, kLine3 = WHICH == 0 ? 31 : 30, kKo = WHICH == 0 ? 27 : 31;
    if (on) {
        const int x = p % kBoard, y = p / kBoard;
        if (x == 2 || x == 16 || y == 2 || y == 16) bits |= 1u << kLine3;
    }
    if (on && c != 2) {
        const bool mine = c == tomove;
        bits |= mine ? 2u : 4u;
        if (extra && c == 1 && moves[(size_t)b * 4 + 3]) bits |= 1u << kKomi;
        const int l = libs[lab[p]];
        if (l >= 1) bits |= 1u << ((mine ? 3 : kOppLib0) + (l >= kLibCap ? kLibCap : l) - 1);
    } else if (on) {
        bits |= 1u;
        int nb[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) nb[k] = nbr(p, k);
        int n_empty_nb = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) n_empty_nb += nb[k] >= 0 && sq[nb[k]] == 2;
        // liberties after a stone of colour col is played here
        int after[2];
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int col = side == 0 ? tomove : !tomove;
            // the strings next to p: joined (own colour) or captured
            // (opponent's with one liberty, which is p); -1 = none
            int join[4], capt[4];
            int join0 = -1;
            bool one_join = true, no_capt = true;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                join[k] = -1;
                capt[k] = -1;
                const int q = nb[k];
                if (q < 0) continue;
                const int cq = sq[q];
                if (cq == col) {
                    join[k] = lab[q];
                    if (join0 < 0) join0 = join[k];
                    else one_join &= join0 == join[k];
                } else if (cq != 2 && libs[lab[q]] == 1) {
                    capt[k] = lab[q];
                    no_capt = false;
                }
            }
            if (no_capt && one_join) {
                // no capture and at most one string joined: the empty
                // neighbours, or the string's liberties less p plus the
                // empty neighbours that are not among them
                int n = n_empty_nb;
                if (join0 >= 0) {
                    n = libs[join0] - 1;
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const int q = nb[k];
                        if (q >= 0 && sq[q] == 2 && !((adj[join0][q >> 5] >> (q & 31)) & 1u)) ++n;
                    }
                }
                after[side] = n;
                continue;
            }
            // words the union can touch: p's neighbours and the joined
            // strings' adjacency sets
            int lo = max(p - kBoard, 0) >> 5, hi = min(p + kBoard, kPoints - 1) >> 5;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (join[k] >= 0) {
                    lo = min(lo, (int)adj_lo[join[k]]);
                    hi = max(hi, (int)adj_hi[join[k]]);
                }
            int n = 0;
            for (int w = lo; w <= hi; ++w) {
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
        if (al >= 1) bits |= 1u << (kAfter0 + (al >= 6 ? 5 : al - 1));
        if (at >= 1) bits |= 1u << (kOAfter0 + (at >= 6 ? 5 : at - 1));
        if (extra && (tomove == 0 || tomove == 1)) {
            int n_empty = 0;
            bool own_atari = false, opp_two = false;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int q = nb[k];
                if (q < 0) continue;
                const int cq = sq[q];
                if (cq == 2) {
                    ++n_empty;
                } else if (cq == 0 || cq == 1) {
                    const int lq = libs[lab[q]];
                    own_atari |= cq == tomove && lq == 1;
                    opp_two |= cq != tomove && lq == 2;
                }
            }
            // ladder: two empty neighbours, an own string in atari next to it
            // (its saving move then is no self-atari)
            if (n_empty == 2 && own_atari) cand[atomicAdd(&ncand, 1)] = (short)p;
            if (opp_two) cand[atomicAdd(&ncand, 1)] = (short)(p | 1 << 9);
        }
    }
    if (extra) {
        __syncthreads();
        // one warp per candidate; the row board in registers (lane y = row y)
        const int lane = p & 31, warp = p >> 5, nwarps = blockDim.x >> 5;
        lad::Board wb;
        wb.c[0] = lane < kBoard ? rowc[0][lane] : 0u;
        wb.c[1] = lane < kBoard ? rowc[1][lane] : 0u;
        const int n = ncand;
        for (int i = warp; i < n; i += nwarps) {
            const int e = cand[i], q = e & 0x1ff;
            if (e >> 9) {
                const bool yes = lad::winning_ladder(wb, tomove, q);
                if (lane == 0) win_yes[q] = yes;
            } else {
                const bool yes = lad::losing_ladder(wb, tomove, q);
                if (lane == 0) lad_yes[q] = yes;
            }
        }
        __syncthreads();
        if (on) {
            if (lad_yes[p]) bits |= 1u << kLadder;
            if (win_yes[p]) bits |= 1u << kWin;
            const int32_t *mv = moves + (size_t)b * 4;
            if (WHICH == 0 && mv[0] == p) bits |= 1u << 28;
            if (WHICH == 0 && mv[0] >= 0 && mv[1] == p) bits |= 1u << 29;
            if (mv[2] == p) bits |= 1u << kKo;
        }
    }
    if (L5) {
        // Row r = y * 19 + x of the board's 399 L5 rows (y = 19, 20: zero
        // pad rows), channel dx * nplanes + c = plane c at (y, x + dx - 2),
        // zero off the board and from channel 5 * nplanes on; 1.0 is `one`.
        // One 16-byte group of 8 channels per thread and step.
        if (on) pbits[p] = bits;
        __syncthreads();
        const int groups = halves * 8;
        uint4 *dst = l5 + (size_t)b * kL5Board * groups;
        const bool aligned = (nplanes & 7) == 0;  // a group's 8 channels share one dx
        if ((int)blockDim.x % groups == 0) {
            // each thread keeps one 16-byte group of channels (their taps dx
            // and planes are constants) and walks the rows: no division by
            // the plane or group count in the loop
            const int g = p % groups, rstep = (int)blockDim.x / groups;
            int dxj[8], cj[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int ch = g * 8 + j;
                dxj[j] = ch / nplanes;
                cj[j] = ch - dxj[j] * nplanes;
            }
            for (int r = p / groups; r < kL5Board; r += rstep) {
                const int y = r / kL5Pitch, x = r - y * kL5Pitch;
                uint32_t w[4] = {0u, 0u, 0u, 0u};
                if (y < kBoard) {
                    if (aligned) {
                        const int sx = x + dxj[0] - 2;
                        if (dxj[0] < 5 && sx >= 0 && sx < kBoard) {
                            const uint32_t v = pbits[y * kBoard + sx] >> cj[0];
#pragma unroll
                            for (int j = 0; j < 4; ++j)
                                w[j] = ((v >> (2 * j)) & 1u) * one | ((v >> (2 * j + 1)) & 1u) * (one << 16);
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int sx = x + dxj[j] - 2;
                            if (dxj[j] < 5 && sx >= 0 && sx < kBoard && ((pbits[y * kBoard + sx] >> cj[j]) & 1u))
                                w[j >> 1] |= (j & 1) ? (one << 16) : one;
                        }
                    }
                }
                dst[(size_t)r * groups + g] = make_uint4(w[0], w[1], w[2], w[3]);
            }
            return;
        }
        for (int i = p; i < kL5Board * groups; i += blockDim.x) {
            const int r = i / groups, g = i - r * groups;
            const int y = r / kL5Pitch, x = r - y * kL5Pitch;
            uint32_t w[4] = {0u, 0u, 0u, 0u};
            if (y < kBoard) {
                if (aligned) {
                    const int ch0 = g * 8, dx = ch0 / nplanes, c0 = ch0 - dx * nplanes, sx = x + dx - 2;
                    if (dx < 5 && sx >= 0 && sx < kBoard) {
                        const uint32_t v = pbits[y * kBoard + sx] >> c0;
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            w[j] = ((v >> (2 * j)) & 1u) * one | ((v >> (2 * j + 1)) & 1u) * (one << 16);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        const int ch = g * 8 + j, dx = ch / nplanes, c = ch - dx * nplanes, sx = x + dx - 2;
                        if (dx < 5 && sx >= 0 && sx < kBoard && ((pbits[y * kBoard + sx] >> c) & 1u))
                            w[j >> 1] |= (j & 1) ? (one << 16) : one;
                    }
                }
            }
            dst[i] = make_uint4(w[0], w[1], w[2], w[3]);
        }
        return;
    }
    if (!on) return;
    uint8_t *dst = planes + (size_t)b * nplanes * kPoints + p;
    for (int i = 0; i < nplanes; ++i) dst[(size_t)i * kPoints] = (uint8_t)((bits >> i) & 1u);
}

// Launched as a programmatic dependent of a trunk, the gather runs on the
// SMs the trunk's CTAs leave (its output must be rows that trunk does not
// read) and waits for the trunk only before it exits, so that a kernel which
// waits for the gather has the trunk's results too.
template <int WHICH, bool EXTRA, bool L5>
__global__ void __launch_bounds__(384, 3) gather_kernel(const int8_t *__restrict__ squares,
                                                     const int8_t *__restrict__ to_move,
                                                     const int32_t *__restrict__ moves, int B,
                                                     int nplanes, uint8_t *__restrict__ planes, int halves,
                                                     uint32_t one, uint4 *__restrict__ l5) {
    ptx::grid_dep_launch();
    gather_board<WHICH, EXTRA, L5>(squares, to_move, moves, B, nplanes, planes, halves, one, l5);
    ptx::grid_dep_wait();
}

template <bool L5>
static void launch_gather_kernel(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B,
                                 int which, int nplanes, uint8_t *planes, int halves, uint32_t one, uint4 *l5,
                                 cudaStream_t s, bool pdl) {
    const bool extra = nplanes > 24;
    void (*k)(const int8_t *, const int8_t *, const int32_t *, int, int, uint8_t *, int, uint32_t, uint4 *) =
        which == 0 ? (extra ? gather_kernel<0, true, L5> : gather_kernel<0, false, L5>)
                   : (extra ? gather_kernel<1, true, L5> : gather_kernel<1, false, L5>);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(B);
    cfg.blockDim = dim3(384);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k, squares, to_move, moves, B, nplanes, planes, halves, one, l5);
}

static int check_gather(int B, int which, int nplanes, const int32_t *moves) {
    if (B < 0 || nplanes < 1 || nplanes > kGatherPlanes || (which != 0 && which != 1) ||
        (nplanes > 24 && !moves && B > 0)) {
        lg_set_error("gather: planes 0..31 of the policy (0) or value (1) set; planes 24..31 need moves");
        return LG_ERR_ARG;
    }
    return LG_OK;
}

int launch_gather(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B, int which,
                  int nplanes, uint8_t *planes, cudaStream_t s, bool pdl) {
    if (int rc = check_gather(B, which, nplanes, moves)) return rc;
    if (B > 0)
        launch_gather_kernel<false>(squares, to_move, moves, B, which, nplanes, planes, 0, 0u, nullptr, s, pdl);
    return LG_OK;
}

int launch_gather_l5(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B, int which,
                     int nplanes, int halves, bool f16, __nv_bfloat16 *l5, cudaStream_t s, bool pdl) {
    if (int rc = check_gather(B, which, nplanes, moves)) return rc;
    if (halves < 1 || 5 * nplanes > halves * 64) {
        lg_set_error("gather: %d planes need %d L5 channels, the layer has %d", nplanes, 5 * nplanes, halves * 64);
        return LG_ERR_ARG;
    }
    if (B > 0)
        launch_gather_kernel<true>(squares, to_move, moves, B, which, nplanes, nullptr, halves,
                                   f16 ? 0x3C00u : 0x3F80u, reinterpret_cast<uint4 *>(l5), s, pdl);
    return LG_OK;
}

}  // namespace lg

extern "C" int lg_gather_device(const int8_t *squares, const int8_t *to_move, const int32_t *moves, int B,
                                int which, int nplanes, uint8_t *planes, void *stream) {
    if ((!squares || !to_move || !planes) && B > 0) {
        lg_set_error("lg_gather_device: bad arguments");
        return LG_ERR_ARG;
    }
    int rc = lg::launch_gather(squares, to_move, moves, B, which, nplanes, planes, (cudaStream_t)stream);
    if (rc) return rc;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        lg_set_error("lg_gather_device: %s", cudaGetErrorString(e));
        return LG_ERR_CUDA;
    }
    return LG_OK;
}
