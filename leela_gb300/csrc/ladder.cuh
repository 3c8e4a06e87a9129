// ladder.cuh -- the ladder reader of the input-plane gather, one warp per
// ladder on row bitboards.
//
// Reference semantics: FastBoard::saving_size (FastBoard.cpp:1273-1292),
// kill_or_connect / self_atari (:1342-1470), is_suicide (:191-240),
// minimum_elib_count (:2429-2442), after_liberties_color (:2511-2528),
// check_winning_ladder (:2530-2564), check_losing_ladder (:2647-2837).  The
// reference keeps incremental string records (parents, liberty counts, stone
// rings); here a board is two colour masks held by a warp, lane y holding
// row y (bit x = point y*19+x; lanes 19..31 hold zeros), and every string,
// liberty count and capture comes from shifts, shuffles and warp votes.  The
// reference's liberty counts are exact, and the two places where it depends
// on the order of a string's liberties (which liberty the attacker tries
// first; the two branches of an even choice) give the same answer in either
// order, so this restatement agrees point for point; the oracle checks it
// against the reference's planes.
//
// Every function here is called by all 32 lanes of a warp with the same
// (warp-uniform) arguments and returns the same value on every lane.
//
// check_losing_ladder recurses on even choices (both ataris tried, result
// OR-ed, at most 5 levels of branching); here that is a depth-first search
// with an explicit stack of at most 6 pending lines, stopping at the first
// losing line.
#pragma once
#include "lg_common.cuh"

namespace lg {
namespace lad {

constexpr unsigned kAll = 0xffffffffu;
constexpr uint32_t kRowBits = (1u << kBoard) - 1;

// this lane's row of black (c[0]) and white (c[1]) stones
struct Board {
    uint32_t c[2];
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t row_mask() { return lane_id() < kBoard ? kRowBits : 0u; }
__device__ __forceinline__ uint32_t point_mask(int p) {
    return lane_id() == p / kBoard ? 1u << (p % kBoard) : 0u;
}
__device__ __forceinline__ uint32_t row_of(uint32_t m, int y) { return __shfl_sync(kAll, m, y); }
__device__ __forceinline__ bool test(uint32_t m, int p) {
    return (row_of(m, p / kBoard) >> (p % kBoard)) & 1u;
}
__device__ __forceinline__ bool any(uint32_t m) { return __any_sync(kAll, m != 0u); }
__device__ __forceinline__ int popc(uint32_t m) {
    return (int)__reduce_add_sync(kAll, (unsigned)__popc(m));
}
// lowest set point of m, or -1
__device__ __forceinline__ int first_point(uint32_t m) {
    const unsigned rows = __ballot_sync(kAll, m != 0u);
    if (!rows) return -1;
    const int y = __ffs(rows) - 1;
    return y * kBoard + __ffs(row_of(m, y)) - 1;
}

__device__ __forceinline__ uint32_t stones(const Board &b, int c) { return c ? b.c[1] : b.c[0]; }
__device__ __forceinline__ void set_stones(Board &b, int c, uint32_t v) {
    if (c) b.c[1] = v;
    else b.c[0] = v;
}
__device__ __forceinline__ uint32_t empties(const Board &b) { return row_mask() & ~(b.c[0] | b.c[1]); }

// the 4-neighbourhood of m (not m itself), on the board
__device__ __forceinline__ uint32_t dilate(uint32_t m) {
    uint32_t up = __shfl_up_sync(kAll, m, 1);
    const uint32_t dn = __shfl_down_sync(kAll, m, 1);
    if (lane_id() == 0) up = 0;
    return ((m << 1) | (m >> 1) | up | dn) & row_mask();
}

// seeds x (inside row r) grown along r towards higher bits: the carry of
// r + x runs from each seed through the set bits above it
__device__ __forceinline__ uint32_t run_up(uint32_t x, uint32_t r) { return (x | ((r + x) ^ r ^ x)) & r; }
// the runs of r that hold a seed of x
__device__ __forceinline__ uint32_t runs_of(uint32_t x, uint32_t r) {
    return run_up(x, r) | __brev(run_up(__brev(x), __brev(r)));
}

// the string of colour-mask `st` through point p (p must be in st): whole
// runs of a row at a time, then a step to the rows above and below
__device__ __forceinline__ uint32_t string_of(uint32_t st, int p) {
    uint32_t s = point_mask(p);
    for (int it = 0; it < 400; ++it) {
        s = runs_of(s, st);
        uint32_t up = __shfl_up_sync(kAll, s, 1);
        const uint32_t dn = __shfl_down_sync(kAll, s, 1);
        if (lane_id() == 0) up = 0;
        const uint32_t n = s | ((up | dn) & st);
        if (!any(n ^ s)) break;
        s = n;
    }
    return s;
}

// liberties of string s (as a mask)
__device__ __forceinline__ uint32_t liberty_mask(const Board &b, uint32_t s) { return dilate(s) & empties(b); }

__device__ __forceinline__ int nbr(int p, int k) {
    const int x = p % kBoard, y = p / kBoard;
    switch (k) {
    case 0: return x > 0 ? p - 1 : -1;
    case 1: return x < kBoard - 1 ? p + 1 : -1;
    case 2: return y > 0 ? p - kBoard : -1;
    default: return y < kBoard - 1 ? p + kBoard : -1;
    }
}

// colour at p: 0, 1, or 2 (empty)
__device__ __forceinline__ int color_at(const Board &b, int p) {
    const int y = p / kBoard, x = p % kBoard;
    const uint32_t r0 = row_of(b.c[0], y), r1 = row_of(b.c[1], y);
    return ((r0 >> x) & 1u) ? 0 : (((r1 >> x) & 1u) ? 1 : 2);
}

// liberties of the string through the stone at p
__device__ __forceinline__ int libs_at(const Board &b, int p) {
    return popc(liberty_mask(b, string_of(stones(b, color_at(b, p)), p)));
}

__device__ __forceinline__ int count_empty_nbrs(const Board &b, int v) {
    const uint32_t e = empties(b);
    const int y = v / kBoard, x = v % kBoard;
    const uint32_t r0 = row_of(e, y);
    const uint32_t ru = row_of(e, y > 0 ? y - 1 : y), rd = row_of(e, y < kBoard - 1 ? y + 1 : y);
    int n = 0;
    if (x > 0) n += (r0 >> (x - 1)) & 1u;
    if (x < kBoard - 1) n += (r0 >> (x + 1)) & 1u;
    if (y > 0) n += (ru >> x) & 1u;
    if (y < kBoard - 1) n += (rd >> x) & 1u;
    return n;
}

// FastBoard::update_board_fast: place, capture opponent strings without
// liberties, remove the new string if it has none
__device__ void play(Board &b, int color, int v) {
    const uint32_t own = stones(b, color) | point_mask(v);
    set_stones(b, color, own);
    uint32_t opp = stones(b, 1 - color);
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0 || !test(opp, q)) continue;
        const uint32_t s = string_of(opp, q);
        if (!any(liberty_mask(b, s))) {
            opp &= ~s;
            set_stones(b, 1 - color, opp);
        }
    }
    const uint32_t s = string_of(own, v);
    if (!any(liberty_mask(b, s))) set_stones(b, color, own & ~s);
}

// FastBoard::minimum_elib_count: fewest liberties among the opponent strings
// next to the point v itself (100 if none)
__device__ int min_elib(const Board &b, int color, int v) {
    int best = 100;
    const uint32_t opp = stones(b, 1 - color);
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0 || !test(opp, q)) continue;
        best = min(best, popc(liberty_mask(b, string_of(opp, q))));
    }
    return best;
}

// FastBoard::is_suicide
__device__ bool is_suicide(const Board &b, int v, int color) {
    if (count_empty_nbrs(b, v) > 0) return false;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0) continue;
        const int cq = color_at(b, q);  // a stone: v has no empty neighbour
        const int l = popc(liberty_mask(b, string_of(stones(b, cq), q)));
        if (cq == color ? l > 1 : l <= 1) return false;
    }
    return true;
}

// FastBoard::self_atari (fewer than two empty neighbours, no capture, no
// connection to 3+ liberties, and v + empty neighbours + liberties of the own
// neighbour strings with 2+ liberties number at most two)
__device__ bool self_atari(const Board &b, int color, int v) {
    if (count_empty_nbrs(b, v) >= 2) return false;
    uint32_t set = point_mask(v);
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0) continue;
        const int c = color_at(b, q);
        if (c == 2) {
            set |= point_mask(q);
            continue;
        }
        const uint32_t l = liberty_mask(b, string_of(stones(b, c), q));
        const int nl = popc(l);
        if ((c == 1 - color && nl <= 1) || (c == color && nl >= 3)) return false;
        if (c == color && nl > 1) set |= l;
    }
    return popc(set) <= 2;
}

// FastBoard::after_liberties_color: liberties of the string formed by playing
// v, 0 for a suicide
__device__ int after_libs(const Board &b, int color, int v) {
    if (is_suicide(b, v, color)) return 0;
    Board t = b;
    play(t, color, v);
    return libs_at(t, v);
}

// the own strings in atari next to vtx: exactly one, which cannot capture
// an attacker (check_losing_ladder's opening tests)
__device__ bool lone_critical_string(const Board &b, int color, int vtx) {
    const uint32_t own = stones(b, color), opp = stones(b, 1 - color);
    uint32_t crit = 0;
    int ncrit = 0;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(vtx, k);
        if (q < 0 || !test(own, q) || test(crit, q)) continue;
        const uint32_t s = string_of(own, q);
        if (popc(liberty_mask(b, s)) > 1) continue;
        ++ncrit;
        crit |= s;
    }
    if (ncrit != 1) return false;
    // any attacker string next to it in atari?
    uint32_t d = dilate(crit) & opp;
    for (int it = 0; it < kPoints; ++it) {
        const int q = first_point(d);
        if (q < 0) break;
        const uint32_t s = string_of(opp, q);
        if (popc(liberty_mask(b, s)) <= 1) return false;
        d &= ~s;
    }
    return true;
}

struct Alt {
    Board b;
    int vtx, branching;
};

// FastBoard::check_losing_ladder(color, vtx): `color` (to move) saves its
// string in atari next to vtx by playing there; true if the attacker can
// keep it in atari until it dies.  Depth-first over the even choices.
__device__ bool losing_ladder(const Board &start, int color, int vtx0) {
    Alt stack[6];
    int top = 0;
    stack[top].b = start;
    stack[top].vtx = vtx0;
    stack[top].branching = 0;
    ++top;
    while (top > 0) {
        --top;
        Board b = stack[top].b;
        const int vtx = stack[top].vtx, branching = stack[top].branching;
        bool result = false;
        if (branching <= 5) {
            const int elib = min_elib(b, color, vtx);
            if (elib != 0 && elib != 1 && lone_critical_string(b, color, vtx)) {
                int atari = vtx;
                play(b, color, vtx);
                for (int step = 0; step < 400; ++step) {
                    const uint32_t own = stones(b, color);
                    if (!test(own, atari)) { result = true; break; }   // the escape was a suicide
                    uint32_t l = liberty_mask(b, string_of(own, atari));
                    const int nl = popc(l);
                    if (nl == 1) { result = true; break; }              // self-atari
                    if (nl >= 3) break;                                  // escaped
                    if (min_elib(b, color, atari) == 1) break;           // counter-atari
                    const int lib0 = first_point(l);
                    l &= ~point_mask(lib0);
                    const int lib1 = first_point(l);
                    if (count_empty_nbrs(b, lib0) == 3 && count_empty_nbrs(b, lib1) == 3) break;
                    int l0 = after_libs(b, color, lib0), l1 = after_libs(b, color, lib1);
                    const bool s0 = is_suicide(b, lib0, 1 - color) || self_atari(b, 1 - color, lib0);
                    const bool s1 = is_suicide(b, lib1, 1 - color) || self_atari(b, 1 - color, lib1);
                    if (s0 && s1) break;
                    if (s0) l1 = l0 + 1;
                    if (s1) l0 = l1 + 1;
                    if (l0 == l1) {
                        // both ataris, each followed by the escape at the
                        // other liberty; lines at branching depth 6 fail at
                        // once, so a depth-5 branch is a failed line (and the
                        // stack holds at most one pending line per depth)
                        if (branching + 1 > 5) break;
                        stack[top].b = b;
                        play(stack[top].b, 1 - color, lib1);
                        stack[top].vtx = lib0;
                        stack[top].branching = branching + 1;
                        ++top;
                        stack[top].b = b;
                        play(stack[top].b, 1 - color, lib0);
                        stack[top].vtx = lib1;
                        stack[top].branching = branching + 1;
                        ++top;
                        break;
                    }
                    play(b, 1 - color, l0 > l1 ? lib0 : lib1);
                    // the string is back in atari: its one liberty is the next saving move
                    l = liberty_mask(b, string_of(stones(b, color), atari));
                    if (popc(l) != 1) break;
                    const int next = first_point(l);
                    play(b, color, next);
                    atari = next;
                }
            }
        }
        if (result) return true;
    }
    return false;
}

// FastBoard::check_winning_ladder(color, vtx)
__device__ bool winning_ladder(const Board &b, int color, int vtx) {
    bool sa_known = false, sa = false;
    const uint32_t opp = stones(b, 1 - color);
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(vtx, k);
        if (q < 0 || !test(opp, q)) continue;
        if (popc(liberty_mask(b, string_of(opp, q))) != 2) continue;
        if (!sa_known) {
            sa = self_atari(b, color, vtx);
            sa_known = true;
        }
        if (sa) continue;
        Board t = b;
        play(t, color, vtx);
        const int esc = first_point(liberty_mask(t, string_of(stones(t, 1 - color), q)));
        if (esc < 0 || count_empty_nbrs(t, esc) != 2) continue;
        if (losing_ladder(t, 1 - color, esc)) return true;
    }
    return false;
}

}  // namespace lad
}  // namespace lg
