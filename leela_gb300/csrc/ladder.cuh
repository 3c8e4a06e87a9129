// ladder.cuh -- the ladder reader of the input-plane gather, on bitboards.
//
// Reference semantics: FastBoard::saving_size (FastBoard.cpp:1273-1292),
// kill_or_connect / self_atari (:1342-1470), is_suicide (:191-240),
// minimum_elib_count (:2429-2442), after_liberties_color (:2511-2528),
// check_winning_ladder (:2530-2564), check_losing_ladder (:2647-2837).  The
// reference keeps incremental string records (parents, liberty counts, stone
// rings); here a board is two 361-bit colour masks (12 words each) and every
// string, liberty count and capture comes from shifts and popcounts, so a
// board copy is 96 bytes.  The reference's liberty counts are exact, and the
// two places where it depends on the order of a string's liberties (which
// liberty the attacker tries first; the two branches of an even choice) give
// the same answer in either order, so this restatement agrees point for
// point; the oracle checks it against the reference's planes.
//
// check_losing_ladder recurses on even choices (both ataris tried, result
// OR-ed, at most 5 levels of branching); here that is a depth-first search
// with an explicit stack of at most 6 pending lines, stopping at the first
// losing line.
#pragma once
#include "lg_common.cuh"

namespace lg {
namespace lad {

constexpr int kW = 12;  // words of a 361-bit mask

struct Masks {
    uint32_t board[kW], notx0[kW], notx18[kW];
};

struct Board {
    uint32_t c[2][kW];  // stones of black (0) and white (1)
};

__device__ __forceinline__ bool test(const uint32_t *m, int p) { return (m[p >> 5] >> (p & 31)) & 1u; }

__device__ __forceinline__ void empties(const Board &b, const Masks &M, uint32_t *e) {
#pragma unroll
    for (int i = 0; i < kW; ++i) e[i] = M.board[i] & ~(b.c[0][i] | b.c[1][i]);
}

// out = the 4-neighbourhood of m (not m itself), on the board
__device__ __forceinline__ void dilate(const uint32_t *m, const Masks &M, uint32_t *out) {
#pragma unroll
    for (int i = 0; i < kW; ++i) {
        const uint32_t e = m[i] & M.notx18[i], w = m[i] & M.notx0[i];
        uint32_t r = (e << 1) | (w >> 1) | (m[i] << 19) | (m[i] >> 19);
        if (i > 0) r |= ((m[i - 1] & M.notx18[i - 1]) >> 31) | (m[i - 1] >> 13);
        if (i < kW - 1) r |= ((m[i + 1] & M.notx0[i + 1]) << 31) | (m[i + 1] << 13);
        out[i] = r & M.board[i];
    }
}

// the string of colour-mask `stones` through point p (p must be in stones)
__device__ __forceinline__ void string_of(const uint32_t *stones, int p, const Masks &M, uint32_t *s) {
#pragma unroll
    for (int i = 0; i < kW; ++i) s[i] = 0;
    s[p >> 5] = 1u << (p & 31);
    for (int it = 0; it < 400; ++it) {
        uint32_t d[kW];
        dilate(s, M, d);
        bool grew = false;
#pragma unroll
        for (int i = 0; i < kW; ++i) {
            const uint32_t n = s[i] | (d[i] & stones[i]);
            grew |= n != s[i];
            s[i] = n;
        }
        if (!grew) break;
    }
}

// liberties of string s (as a mask)
__device__ __forceinline__ void liberty_mask(const Board &b, const uint32_t *s, const Masks &M, uint32_t *l) {
    uint32_t e[kW];
    empties(b, M, e);
    dilate(s, M, l);
#pragma unroll
    for (int i = 0; i < kW; ++i) l[i] &= e[i];
}

__device__ __forceinline__ int popc(const uint32_t *m) {
    int n = 0;
#pragma unroll
    for (int i = 0; i < kW; ++i) n += __popc(m[i]);
    return n;
}

// lowest set point of m, or -1
__device__ __forceinline__ int first_point(const uint32_t *m) {
#pragma unroll
    for (int i = 0; i < kW; ++i)
        if (m[i]) return i * 32 + __ffs(m[i]) - 1;
    return -1;
}

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
    return test(b.c[0], p) ? 0 : (test(b.c[1], p) ? 1 : 2);
}

__device__ __forceinline__ int libs_at(const Board &b, int p, const Masks &M) {
    uint32_t s[kW], l[kW];
    string_of(b.c[color_at(b, p)], p, M, s);
    liberty_mask(b, s, M, l);
    return popc(l);
}

__device__ __forceinline__ int count_empty_nbrs(const Board &b, int v) {
    int n = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q >= 0 && color_at(b, q) == 2) ++n;
    }
    return n;
}

__device__ __forceinline__ void clear(uint32_t *dst, const uint32_t *s) {
#pragma unroll
    for (int i = 0; i < kW; ++i) dst[i] &= ~s[i];
}

// FastBoard::update_board_fast: place, capture opponent strings without
// liberties, remove the new string if it has none
__device__ void play(Board &b, int color, int v, const Masks &M) {
    b.c[color][v >> 5] |= 1u << (v & 31);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0 || !test(b.c[1 - color], q)) continue;
        uint32_t s[kW], l[kW];
        string_of(b.c[1 - color], q, M, s);
        liberty_mask(b, s, M, l);
        if (popc(l) == 0) clear(b.c[1 - color], s);
    }
    uint32_t s[kW], l[kW];
    string_of(b.c[color], v, M, s);
    liberty_mask(b, s, M, l);
    if (popc(l) == 0) clear(b.c[color], s);
}

// FastBoard::minimum_elib_count: fewest liberties among the opponent strings
// next to the point v itself (100 if none)
__device__ int min_elib(const Board &b, int color, int v, const Masks &M) {
    int best = 100;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0 || !test(b.c[1 - color], q)) continue;
        best = min(best, libs_at(b, q, M));
    }
    return best;
}

// FastBoard::is_suicide
__device__ bool is_suicide(const Board &b, int v, int color, const Masks &M) {
    if (count_empty_nbrs(b, v) > 0) return false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0) continue;
        const int l = libs_at(b, q, M);
        if (color_at(b, q) == color ? l > 1 : l <= 1) return false;
    }
    return true;
}

// FastBoard::self_atari (fewer than two empty neighbours, no capture, no
// connection to 3+ liberties, and v + empty neighbours + liberties of the own
// neighbour strings with 2+ liberties number at most two)
__device__ bool self_atari(const Board &b, int color, int v, const Masks &M) {
    if (count_empty_nbrs(b, v) >= 2) return false;
    uint32_t set[kW];
#pragma unroll
    for (int i = 0; i < kW; ++i) set[i] = 0;
    set[v >> 5] |= 1u << (v & 31);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(v, k);
        if (q < 0) continue;
        const int c = color_at(b, q);
        if (c == 2) {
            set[q >> 5] |= 1u << (q & 31);
            continue;
        }
        uint32_t s[kW], l[kW];
        string_of(b.c[c], q, M, s);
        liberty_mask(b, s, M, l);
        const int nl = popc(l);
        if ((c == 1 - color && nl <= 1) || (c == color && nl >= 3)) return false;
        if (c == color && nl > 1)
#pragma unroll
            for (int i = 0; i < kW; ++i) set[i] |= l[i];
    }
    return popc(set) <= 2;
}

// FastBoard::after_liberties_color: liberties of the string formed by playing
// v, 0 for a suicide
__device__ int after_libs(const Board &b, int color, int v, const Masks &M) {
    if (is_suicide(b, v, color, M)) return 0;
    Board t = b;
    play(t, color, v, M);
    return libs_at(t, v, M);
}

// the own strings in atari next to vtx: exactly one, which cannot capture
// an attacker (check_losing_ladder's opening tests)
__device__ bool lone_critical_string(const Board &b, int color, int vtx, const Masks &M) {
    uint32_t crit[kW];
    int ncrit = 0;
#pragma unroll
    for (int i = 0; i < kW; ++i) crit[i] = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(vtx, k);
        if (q < 0 || !test(b.c[color], q) || test(crit, q)) continue;
        uint32_t s[kW], l[kW];
        string_of(b.c[color], q, M, s);
        liberty_mask(b, s, M, l);
        if (popc(l) > 1) continue;
        ++ncrit;
#pragma unroll
        for (int i = 0; i < kW; ++i) crit[i] |= s[i];
    }
    if (ncrit != 1) return false;
    // any attacker string next to it in atari?
    uint32_t d[kW];
    dilate(crit, M, d);
#pragma unroll
    for (int i = 0; i < kW; ++i) d[i] &= b.c[1 - color][i];
    while (true) {
        const int q = first_point(d);
        if (q < 0) break;
        uint32_t s[kW], l[kW];
        string_of(b.c[1 - color], q, M, s);
        liberty_mask(b, s, M, l);
        if (popc(l) <= 1) return false;
        clear(d, s);
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
__device__ bool losing_ladder(const Board &start, int color, int vtx0, const Masks &M) {
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
            const int elib = min_elib(b, color, vtx, M);
            if (elib != 0 && elib != 1 && lone_critical_string(b, color, vtx, M)) {
                int atari = vtx;
                play(b, color, vtx, M);
                for (int step = 0; step < 400; ++step) {
                    if (!test(b.c[color], atari)) { result = true; break; }   // the escape was a suicide
                    uint32_t s[kW], l[kW];
                    string_of(b.c[color], atari, M, s);
                    liberty_mask(b, s, M, l);
                    const int nl = popc(l);
                    if (nl == 1) { result = true; break; }                      // self-atari
                    if (nl >= 3) break;                                          // escaped
                    if (min_elib(b, color, atari, M) == 1) break;                // counter-atari
                    const int lib0 = first_point(l);
                    l[lib0 >> 5] &= ~(1u << (lib0 & 31));
                    const int lib1 = first_point(l);
                    if (count_empty_nbrs(b, lib0) == 3 && count_empty_nbrs(b, lib1) == 3) break;
                    int l0 = after_libs(b, color, lib0, M), l1 = after_libs(b, color, lib1, M);
                    const bool s0 = is_suicide(b, lib0, 1 - color, M) || self_atari(b, 1 - color, lib0, M);
                    const bool s1 = is_suicide(b, lib1, 1 - color, M) || self_atari(b, 1 - color, lib1, M);
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
                        play(stack[top].b, 1 - color, lib1, M);
                        stack[top].vtx = lib0;
                        stack[top].branching = branching + 1;
                        ++top;
                        stack[top].b = b;
                        play(stack[top].b, 1 - color, lib0, M);
                        stack[top].vtx = lib1;
                        stack[top].branching = branching + 1;
                        ++top;
                        break;
                    }
                    play(b, 1 - color, l0 > l1 ? lib0 : lib1, M);
                    // the string is back in atari: its one liberty is the next saving move
                    string_of(b.c[color], atari, M, s);
                    liberty_mask(b, s, M, l);
                    if (popc(l) != 1) break;
                    const int next = first_point(l);
                    play(b, color, next, M);
                    atari = next;
                }
            }
        }
        if (result) return true;
    }
    return false;
}

// FastBoard::check_winning_ladder(color, vtx)
__device__ bool winning_ladder(const Board &b, int color, int vtx, const Masks &M) {
    bool sa_known = false, sa = false;
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        const int q = nbr(vtx, k);
        if (q < 0 || !test(b.c[1 - color], q)) continue;
        uint32_t s[kW], l[kW];
        string_of(b.c[1 - color], q, M, s);
        liberty_mask(b, s, M, l);
        if (popc(l) != 2) continue;
        if (!sa_known) {
            sa = self_atari(b, color, vtx, M);
            sa_known = true;
        }
        if (sa) continue;
        Board t = b;
        play(t, color, vtx, M);
        string_of(t.c[1 - color], q, M, s);
        liberty_mask(t, s, M, l);
        const int esc = first_point(l);
        if (esc < 0 || count_empty_nbrs(t, esc) != 2) continue;
        if (losing_ladder(t, 1 - color, esc, M)) return true;
    }
    return false;
}

}  // namespace lad
}  // namespace lg
