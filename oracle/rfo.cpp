/*
 * rfo.cpp -- CPU oracle for the bit-parallel string scorers (TEST INFRASTRUCTURE ONLY).
 *
 * A restatement of rapidfuzz-cpp v3.3.3 (paths below are relative to that project):
 *   - pattern-match vectors           rapidfuzz/details/PatternMatchVector.hpp:62-221
 *   - Levenshtein (Hyyro 2003, band, Myers block, dispatch, weights)
 *                                     rapidfuzz/distance/Levenshtein_impl.hpp:85-155, 259-322, 419-505,
 *                                     641-905, 1056-1089
 *   - LCSseq / Indel (Hyyro 2004)     rapidfuzz/distance/LCSseq_impl.hpp:205-403, Indel_impl.hpp:14-66
 *   - OSA (Hyyro 2003 + transpositions) rapidfuzz/distance/OSA_impl.hpp:34-74, 176-273, OSA.hpp:253-267
 *   - Jaro / Jaro-Winkler             rapidfuzz/distance/Jaro_impl.hpp:32-454, JaroWinkler_impl.hpp:9-71
 *   - formula chains of the bases     rapidfuzz/details/distance.hpp:52-76, 120-133, 177-203, 240-262,
 *                                     304-317, 359-369, 421-460, 500-512, 552-563; common.hpp:50-53
 *   - Multi* batch scorers            Levenshtein.hpp:297-419, LCSseq.hpp:77-195, Indel.hpp:77-146,
 *                                     OSA.hpp:113-230, Jaro.hpp:64-193, JaroWinkler.hpp:75-166
 *   - fuzz::ratio                     rapidfuzz/fuzz_impl.hpp:22-47, fuzz.hpp:50-95
 *   - naive DP oracles                rapidfuzz_reference/{Levenshtein,LCSseq,OSA,Jaro}.hpp
 *
 * Two shortcuts of the reference are replaced by the bit-parallel paths they shortcut:
 * mbleven (Levenshtein cutoff < 4, LCS max_misses < 5) and common-affix stripping.  Both
 * return the same value under the cutoff contract d <= c ? d : c+1 (resp. s >= c ? s : 0),
 * which the tests check against the reference itself.
 *
 * Build with -ffp-contract=off: the double formulas must not be fused into FMAs.
 */
#include "rfo.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

typedef uint64_t u64;
typedef int64_t i64;

inline int popc(u64 x) { return __builtin_popcountll(x); }
inline int ctz(u64 x) { return __builtin_ctzll(x); }
inline u64 blsi(u64 x) { return x & (0 - x); }
inline u64 blsr(u64 x) { return x & (x - 1); }
inline i64 absdiff(i64 a, i64 b) { return a > b ? a - b : b - a; }
inline i64 ceil_div(i64 a, i64 d) { return a / d + (a % d != 0); }
inline u64 ceil_div_u(u64 a, u64 d) { return a / d + (a % d != 0); }

/* ------------------------------------------------------------------ strings */

template <typename C>
struct Str {
    const C* p;
    i64 n;
    u64 operator[](i64 i) const { return (u64)p[i]; }
};

/* call f(Str<C1>, Str<C2>) with the code-unit types named by the widths */
template <typename F>
auto with_strs(const void* a, i64 la, int ca, const void* b, i64 lb, int cb, F f) -> decltype(
    f(Str<uint8_t>{nullptr, 0}, Str<uint8_t>{nullptr, 0}))
{
#define RFO_B(CA, TA)                                                                   \
    switch (cb) {                                                                       \
    case 1: return f(Str<TA>{(const TA*)a, la}, Str<uint8_t>{(const uint8_t*)b, lb});   \
    case 2: return f(Str<TA>{(const TA*)a, la}, Str<uint16_t>{(const uint16_t*)b, lb}); \
    case 4: return f(Str<TA>{(const TA*)a, la}, Str<uint32_t>{(const uint32_t*)b, lb}); \
    default: return f(Str<TA>{(const TA*)a, la}, Str<uint64_t>{(const uint64_t*)b, lb}); \
    }
    switch (ca) {
    case 1: RFO_B(1, uint8_t)
    case 2: RFO_B(2, uint16_t)
    case 4: RFO_B(4, uint32_t)
    default: RFO_B(8, uint64_t)
    }
#undef RFO_B
}

template <typename S1, typename S2>
bool str_equal(const S1& a, const S2& b)
{
    if (a.n != b.n) return false;
    for (i64 i = 0; i < a.n; ++i)
        if (a[i] != b[i]) return false;
    return true;
}

/* ------------------------------------------------------- pattern-match vectors
 * PM[c] bit i (word i/64) is set when s1[i] == c.  Code units below 256 index a
 * dense table; larger ones go through an open-addressing table (PatternMatchVector.hpp:62-221
 * uses a 128-slot CPython-probing map per word for these; a linear-probing table
 * holds the same sets). */
struct PM {
    i64 words = 0;
    std::vector<u64> lo; /* [256][words] */
    u64 cap = 0;         /* power of two, or 0 */
    std::vector<u64> keys;
    std::vector<u64> vals; /* [cap][words] */

    static u64 slot_of(u64 c, u64 cap) { return (c * 0x9E3779B97F4A7C15ull) >> 20 & (cap - 1); }

    template <typename S>
    void build(const S& s)
    {
        words = ceil_div(s.n, 64);
        lo.assign(256 * (size_t)std::max<i64>(words, 1), 0);
        i64 hi = 0;
        for (i64 i = 0; i < s.n; ++i)
            hi += s[i] >= 256;
        cap = 0;
        if (hi) {
            cap = 8;
            while (cap < (u64)(2 * hi)) cap <<= 1;
            keys.assign(cap, 0);
            vals.assign(cap * (size_t)words, 0);
        }
        for (i64 i = 0; i < s.n; ++i) {
            u64 c = s[i];
            u64 bit = 1ull << (i % 64);
            if (c < 256) {
                lo[c * words + i / 64] |= bit;
            }
            else {
                u64 k = slot_of(c, cap);
                while (keys[k] != 0 && keys[k] != c) k = (k + 1) & (cap - 1);
                keys[k] = c;
                vals[k * words + i / 64] |= bit;
            }
        }
    }

    u64 get(i64 w, u64 c) const
    {
        if (c < 256) return lo[c * words + w];
        if (!cap) return 0;
        u64 k = slot_of(c, cap);
        while (true) {
            if (keys[k] == c) return vals[k * words + w];
            if (keys[k] == 0) return 0;
            k = (k + 1) & (cap - 1);
        }
    }
};

/* ================================================================ Levenshtein */

/* single word, s1 length 1..64 (Levenshtein_impl.hpp:259-322) */
template <typename S2>
i64 lev_hyyro_word(const PM& pm, i64 m, const S2& t)
{
    u64 VP = ~0ull, VN = 0;
    i64 dist = m;
    const u64 top = 1ull << (m - 1);
    for (i64 j = 0; j < t.n; ++j) {
        u64 X = pm.get(0, t[j]);
        u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
        u64 HP = VN | ~(D0 | VP);
        u64 HN = D0 & VP;
        dist += (HP & top) != 0;
        dist -= (HN & top) != 0;
        HP = (HP << 1) | 1;
        HN = HN << 1;
        VP = HN | ~(D0 | HP);
        VN = HP & D0;
    }
    return dist;
}

/* diagonal band of one word, 2*max+1 <= 64, s1 > 64 (Levenshtein_impl.hpp:419-505) */
template <typename S2>
i64 lev_small_band(const PM& pm, i64 m, const S2& t, i64 max)
{
    u64 VP = ~0ull << (64 - max - 1);
    u64 VN = 0;
    const i64 words = pm.words;
    i64 dist = max;
    const u64 diag = 1ull << 63;
    u64 horiz = 1ull << 62;
    i64 start = max + 1 - 64;
    const i64 break_score = 2 * max + t.n - m;

    auto pm_window = [&](u64 c) -> u64 {
        if (start < 0) return pm.get(0, c) << (-start);
        i64 w = start / 64, b = start % 64;
        u64 x = pm.get(w, c) >> b;
        if (w + 1 < words && b != 0) x |= pm.get(w + 1, c) << (64 - b);
        return x;
    };

    i64 j = 0;
    if (m > max) {
        for (; j < m - max; ++j, ++start) {
            u64 X = pm_window(t[j]);
            u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
            u64 HP = VN | ~(D0 | VP);
            u64 HN = D0 & VP;
            dist += (D0 & diag) == 0;
            if (dist > break_score) return max + 1;
            VP = HN | ~((D0 >> 1) | HP);
            VN = (D0 >> 1) & HP;
        }
    }
    for (; j < t.n; ++j, ++start) {
        u64 X = pm_window(t[j]);
        u64 D0 = (((X & VP) + VP) ^ VP) | X | VN;
        u64 HP = VN | ~(D0 | VP);
        u64 HN = D0 & VP;
        dist += (HP & horiz) != 0;
        dist -= (HN & horiz) != 0;
        horiz >>= 1;
        if (dist > break_score) return max + 1;
        VP = HN | ~((D0 >> 1) | HP);
        VN = (D0 >> 1) & HP;
    }
    return dist <= max ? dist : max + 1;
}

/* Myers/Hyyro multi-word with the Ukkonen band of the reference (Levenshtein_impl.hpp:641-850) */
template <typename S2>
i64 lev_block(const PM& pm, i64 m, const S2& t, i64 max)
{
    const i64 n = t.n;
    if (max < absdiff(m, n)) return max + 1;
    const i64 words = pm.words;
    std::vector<u64> VP(words, ~0ull), VN(words, 0);
    std::vector<i64> score(words);
    const u64 last = 1ull << ((m - 1) % 64);
    for (i64 w = 0; w < words - 1; ++w) score[w] = (w + 1) * 64;
    score[words - 1] = m;

    max = std::min(max, std::max(m, n));
    i64 first = 0;
    i64 lastb = std::min(words, ceil_div(std::min(max, (max + m - n) / 2) + 1, 64)) - 1;

    auto row_of = [&](i64 w) -> i64 { return (w + 1 == words) ? m - 1 : (w + 1) * 64 - 1; };

    for (i64 row = 0; row < n; ++row) {
        const u64 c = t[row];
        u64 hp_carry = 1, hn_carry = 0;
        auto advance = [&](i64 w) -> i64 {
            u64 X = pm.get(w, c) | hn_carry;
            u64 vp = VP[w], vn = VN[w];
            u64 D0 = (((X & vp) + vp) ^ vp) | X | vn;
            u64 HP = vn | ~(D0 | vp);
            u64 HN = D0 & vp;
            u64 hp_in = hp_carry, hn_in = hn_carry;
            if (w < words - 1) {
                hp_carry = HP >> 63;
                hn_carry = HN >> 63;
            }
            else {
                hp_carry = (HP & last) != 0;
                hn_carry = (HN & last) != 0;
            }
            HP = (HP << 1) | hp_in;
            HN = (HN << 1) | hn_in;
            VP[w] = HN | ~(D0 | HP);
            VN[w] = HP & D0;
            return (i64)hp_carry - (i64)hn_carry;
        };

        for (i64 w = first; w <= lastb; ++w) score[w] += advance(w);

        max = std::min(max, score[lastb] + std::max(n - row - 1, m - (1 + lastb) * 64 + 2));

        if (lastb + 1 < words) {
            i64 cond = (max + 128 + row + m) - (score[lastb] + 2 + n);
            if (row_of(lastb) < cond) {
                ++lastb;
                VP[lastb] = ~0ull;
                VN[lastb] = 0;
                i64 chars = (lastb + 1 == words) ? ((m - 1) % 64 + 1) : 64;
                score[lastb] = score[lastb - 1] + chars - (i64)hp_carry + (i64)hn_carry;
                score[lastb] += advance(lastb);
            }
        }
        for (; lastb >= first; --lastb) {
            bool c1 = score[lastb] < max + 64;
            i64 cond = (max + 128 + row + m + 1) - (score[lastb] + 2 + n);
            bool c2 = row_of(lastb) <= cond;
            if (c1 && c2) break;
        }
        for (; first <= lastb; ++first) {
            bool c1 = score[first] < max + 64;
            i64 cond = (score[first] + m + row) - (max + n);
            bool c2 = row_of(first) >= cond;
            if (c1 && c2) break;
        }
        if (lastb < first) return max + 1;
    }
    i64 dist = score[words - 1];
    return dist > max ? max + 1 : dist;
}

/* uniform Levenshtein with a cached pattern (Levenshtein_impl.hpp:852-905) */
template <typename S1, typename S2>
u64 lev_uniform_cached(const PM& pm, const S1& s1, const S2& s2, u64 cutoff, u64 hint)
{
    const i64 m = s1.n, n = s2.n;
    cutoff = std::min<u64>(cutoff, (u64)std::max(m, n));
    if (hint < 31) hint = 31;
    if (cutoff == 0) return str_equal(s1, s2) ? 0 : 1;
    if (cutoff < (u64)absdiff(m, n)) return cutoff + 1;
    if (m == 0) return (u64)n <= cutoff ? (u64)n : cutoff + 1;
    const i64 k = (i64)cutoff;
    if (m < 65) {
        i64 d = lev_hyyro_word(pm, m, s2);
        return d <= k ? (u64)d : cutoff + 1;
    }
    if (cutoff >= 4) {
        if (std::min<i64>(m, 2 * k + 1) <= 64) return (u64)lev_small_band(pm, m, s2, k);
        while (hint < cutoff) {
            i64 h = (i64)hint;
            i64 s = std::min<i64>(m, 2 * h + 1) <= 64 ? lev_small_band(pm, m, s2, h) : lev_block(pm, m, s2, h);
            if (s <= h) return (u64)s;
            if (std::numeric_limits<u64>::max() / 2 < hint) break;
            hint *= 2;
        }
    }
    return (u64)lev_block(pm, m, s2, k);
}

/* LCS: Hyyro 2004 full (LCSseq_impl.hpp:205-260) and banded (:262-333) */
template <typename S2>
i64 lcs_full(const PM& pm, const S2& t)
{
    const i64 words = pm.words;
    if (words == 1) { /* one word in a register, as lcs_unroll<1> (LCSseq_impl.hpp:205-260) */
        u64 S = ~0ull;
        for (i64 j = 0; j < t.n; ++j) {
            const u64 u = S & pm.get(0, t[j]);
            S = (S + u) | (S - u);
        }
        return popc(~S);
    }
    std::vector<u64> S(words, ~0ull);
    for (i64 j = 0; j < t.n; ++j) {
        const u64 c = t[j];
        u64 carry = 0;
        for (i64 w = 0; w < words; ++w) {
            u64 M = pm.get(w, c);
            u64 u = S[w] & M;
            u64 x = S[w] + u;
            u64 c1 = x < u;
            u64 x2 = x + carry;
            u64 c2 = x2 < carry;
            carry = c1 | c2;
            S[w] = x2 | (S[w] - u);
        }
    }
    i64 sim = 0;
    for (i64 w = 0; w < words; ++w) sim += popc(~S[w]);
    return sim;
}

template <typename S2>
i64 lcs_blockwise(const PM& pm, i64 m, const S2& t, i64 cutoff)
{
    const i64 words = pm.words;
    std::vector<u64> S(words, ~0ull);
    const i64 left = m - cutoff, right = t.n - cutoff;
    i64 first = 0, last = std::min(words, ceil_div(left + 1, 64));
    for (i64 row = 0; row < t.n; ++row) {
        const u64 c = t[row];
        u64 carry = 0;
        for (i64 w = first; w < last; ++w) {
            u64 M = pm.get(w, c);
            u64 s = S[w];
            u64 u = s & M;
            u64 x = s + u;
            u64 c1 = x < u;
            u64 x2 = x + carry;
            u64 c2 = x2 < carry;
            carry = c1 | c2;
            S[w] = x2 | (s - u);
        }
        if (row > right) first = (row - right) / 64;
        if (row + 1 + left <= m) last = ceil_div(row + 1 + left, 64);
    }
    i64 sim = 0;
    for (u64 s : S) sim += popc(~s);
    return sim;
}

/* lcs_seq_similarity with a cached pattern (LCSseq_impl.hpp:335-403) */
template <typename S1, typename S2>
u64 lcs_cached(const PM& pm, const S1& s1, const S2& s2, u64 cutoff)
{
    const i64 m = s1.n, n = s2.n;
    if (cutoff > (u64)m || cutoff > (u64)n) return 0;
    const i64 c = (i64)cutoff;
    const i64 max_misses = m + n - 2 * c;
    if (max_misses == 0 || (max_misses == 1 && m == n)) return str_equal(s1, s2) ? (u64)m : 0;
    if (max_misses < absdiff(m, n)) return 0;
    if (m == 0) return 0;
    /* max_misses < 5 goes through affix stripping + mbleven in the reference (exact under
     * the cutoff); the unbanded run gives the same value.  The banded run is only taken
     * where the reference takes it. */
    const i64 full_band = (m - c) + 1 + (n - c);
    const i64 fbw = std::min(pm.words, full_band / 64 + 2);
    i64 sim = (max_misses >= 5 && fbw < pm.words) ? lcs_blockwise(pm, m, s2, c) : lcs_full(pm, s2);
    return sim >= c ? (u64)sim : 0;
}

/* ======================================================================== OSA */

template <typename S2>
i64 osa_word(const PM& pm, i64 m, const S2& t)
{
    u64 VP = ~0ull, VN = 0, D0 = 0, PMold = 0;
    i64 dist = m;
    const u64 top = 1ull << (m - 1);
    for (i64 j = 0; j < t.n; ++j) {
        u64 X = pm.get(0, t[j]);
        u64 TR = (((~D0) & X) << 1) & PMold;
        D0 = (((X & VP) + VP) ^ VP) | X | VN;
        D0 |= TR;
        u64 HP = VN | ~(D0 | VP);
        u64 HN = D0 & VP;
        dist += (HP & top) != 0;
        dist -= (HN & top) != 0;
        HP = (HP << 1) | 1;
        HN = HN << 1;
        VP = HN | ~(D0 | HP);
        VN = HP & D0;
        PMold = X;
    }
    return dist;
}

template <typename S2>
i64 osa_block(const PM& pm, i64 m, const S2& t)
{
    struct Row {
        u64 VP = ~0ull, VN = 0, D0 = 0, PM = 0;
    };
    const i64 words = pm.words;
    const u64 last = 1ull << ((m - 1) % 64);
    i64 dist = m;
    std::vector<Row> oldr(words + 1), newr(words + 1);
    for (i64 j = 0; j < t.n; ++j) {
        const u64 c = t[j];
        u64 hp_carry = 1, hn_carry = 0;
        for (i64 w = 0; w < words; ++w) {
            u64 VN = oldr[w + 1].VN, VP = oldr[w + 1].VP, D0 = oldr[w + 1].D0;
            u64 D0_prev_word = oldr[w].D0;
            u64 PM_old = oldr[w + 1].PM;
            u64 PM_prev_word = newr[w].PM;
            u64 X = pm.get(w, c);
            u64 TR = ((((~D0) & X) << 1) | (((~D0_prev_word) & PM_prev_word) >> 63)) & PM_old;
            u64 Xc = X | hn_carry;
            D0 = (((Xc & VP) + VP) ^ VP) | Xc | VN | TR;
            u64 HP = VN | ~(D0 | VP);
            u64 HN = D0 & VP;
            if (w == words - 1) {
                dist += (HP & last) != 0;
                dist -= (HN & last) != 0;
            }
            u64 hp_in = hp_carry;
            hp_carry = HP >> 63;
            HP = (HP << 1) | hp_in;
            u64 hn_in = hn_carry;
            hn_carry = HN >> 63;
            HN = (HN << 1) | hn_in;
            newr[w + 1].VP = HN | ~(D0 | HP);
            newr[w + 1].VN = HP & D0;
            newr[w + 1].D0 = D0;
            newr[w + 1].PM = X;
        }
        std::swap(newr, oldr);
    }
    return dist;
}

/* CachedOSA::_distance (OSA.hpp:253-267) */
template <typename S1, typename S2>
u64 osa_cached(const PM& pm, const S1& s1, const S2& s2, u64 cutoff)
{
    u64 res;
    if (s1.n == 0) res = (u64)s2.n;
    else if (s2.n == 0) res = (u64)s1.n;
    else if (s1.n < 64) res = (u64)osa_word(pm, s1.n, s2);
    else res = (u64)osa_block(pm, s1.n, s2);
    return res <= cutoff ? res : cutoff + 1;
}

/* ======================================================================= Jaro */

/* greedy flagging over words (Jaro_impl.hpp:94-315): every text character takes
 * the first unflagged equal pattern character inside its window */
template <typename S1, typename S2>
void jaro_counts_pm(const PM& pm, const S1& P, const S2& T, i64* common, i64* transp)
{
    const i64 pl = P.n, tl = T.n;
    *common = 0;
    *transp = 0;
    if (!pl || !tl) return;
    i64 bound = std::max(pl, tl) / 2;
    if (bound > 0) --bound;
    const i64 pw = pm.words;
    std::vector<u64> pflag(pw, 0), tflag(ceil_div(tl, 64), 0);
    for (i64 j = 0; j < tl; ++j) {
        i64 lo = j >= bound ? j - bound : 0;
        i64 hi = std::min(j + bound, pl - 1);
        if (lo > hi) continue;
        const u64 c = T[j];
        for (i64 w = lo / 64; w <= hi / 64; ++w) {
            u64 mask = ~0ull;
            if (w == lo / 64) mask &= ~0ull << (lo % 64);
            if (w == hi / 64) mask &= (hi % 64 == 63) ? ~0ull : ((1ull << (hi % 64 + 1)) - 1);
            u64 x = pm.get(w, c) & mask & ~pflag[w];
            if (x) {
                pflag[w] |= blsi(x);
                tflag[j / 64] |= 1ull << (j % 64);
                break;
            }
        }
    }
    i64 cc = 0;
    for (u64 f : pflag) cc += popc(f);
    *common = cc;
    i64 pwi = 0;
    u64 pf = pflag.empty() ? 0 : pflag[0];
    i64 t = 0;
    for (i64 tw = 0; tw < (i64)tflag.size(); ++tw) {
        u64 tf = tflag[tw];
        while (tf) {
            while (!pf) pf = pflag[++pwi];
            i64 j = tw * 64 + ctz(tf);
            u64 bit = blsi(pf);
            t += (pm.get(pwi, T[j]) & bit) == 0;
            tf = blsr(tf);
            pf ^= bit;
        }
    }
    *transp = t;
}

double jaro_formula(i64 pl, i64 tl, i64 common, i64 transp)
{
    transp /= 2;
    double sim = 0;
    sim += (double)common / (double)pl;
    sim += (double)common / (double)tl;
    sim += ((double)common - (double)transp) / (double)common;
    return sim / 3.0;
}

bool jaro_length_filter(i64 pl, i64 tl, double cutoff)
{
    if (!tl || !pl) return false;
    double mn = (double)std::min(pl, tl);
    double sim = mn / (double)pl + mn / (double)tl + 1.0;
    sim /= 3.0;
    return sim >= cutoff;
}

bool jaro_common_filter(i64 pl, i64 tl, i64 common, double cutoff)
{
    if (!common) return false;
    double sim = 0;
    sim += (double)common / (double)pl;
    sim += (double)common / (double)tl;
    sim += 1.0;
    sim /= 3.0;
    return sim >= cutoff;
}

/* jaro_similarity (Jaro_impl.hpp:409-454) with its filters, from exact counts */
double jaro_from_counts(i64 pl, i64 tl, i64 common, i64 transp, double cutoff)
{
    if (cutoff > 1.0) return 0.0;
    if (!pl && !tl) return 1.0;
    if (!jaro_length_filter(pl, tl, cutoff)) return 0.0;
    if (pl == 1 && tl == 1) return (double)(common == 1);
    if (!jaro_common_filter(pl, tl, common, cutoff)) return 0.0;
    double sim = jaro_formula(pl, tl, common, transp);
    return sim >= cutoff ? sim : 0;
}

template <typename S1, typename S2>
i64 common_prefix4(const S1& P, const S2& T)
{
    i64 mx = std::min<i64>(std::min(P.n, T.n), 4);
    i64 k = 0;
    for (; k < mx; ++k)
        if (T[k] != P[k]) break;
    return k;
}

/* jaro_winkler_similarity (JaroWinkler_impl.hpp:41-71) */
template <typename JaroFn>
double jw_chain(i64 prefix, double pw, double cutoff, JaroFn jaro)
{
    double jc = cutoff;
    if (jc > 0.7) {
        double ps = (double)prefix * pw;
        if (ps >= 1.0) jc = 0.7;
        else jc = std::max(0.7, (ps - jc) / (ps - 1.0));
    }
    double sim = jaro(jc);
    if (sim > 0.7) {
        sim += (double)prefix * pw * (1.0 - sim);
        sim = std::min(sim, 1.0);
    }
    return sim >= cutoff ? sim : 0;
}

/* MultiJaro (jaro_similarity_simd, Jaro_impl.hpp:818-840, 666-709) from exact counts */
double multi_jaro_from_counts(i64 pl, i64 tl, i64 common, i64 transp, double cutoff)
{
    if (cutoff > 1.0) return 0.0;
    if (tl == 0) return pl ? 0.0 : 1.0;
    if (!jaro_common_filter(pl, tl, common, cutoff)) return 0.0;
    double sim = jaro_formula(pl, tl, common, transp);
    return sim >= cutoff ? sim : 0;
}

/* MultiJaroWinkler::_similarity (JaroWinkler.hpp:123-145) */
double multi_jw(double jaro_sim, i64 prefix, double pw, double cutoff)
{
    double s = jaro_sim;
    if (s > 0.7) {
        s += (double)prefix * pw * (1.0 - s);
        s = std::min(s, 1.0);
    }
    if (s < cutoff) s = 0.0;
    return s;
}

/* ============================================================ formula chains */

inline double norm_sim_to_norm_dist(double c) { return std::min(1.0, 1.0 - c + 0.00001); }

u64 lev_maximum(u64 l1, u64 l2, const rfo_params* w)
{
    u64 ins = (u64)w->insert_cost, del = (u64)w->delete_cost, rep = (u64)w->replace_cost;
    u64 mx = l1 * del + l2 * ins;
    if (l1 >= l2) mx = std::min(mx, l2 * rep + (l1 - l2) * del);
    else mx = std::min(mx, l1 * rep + (l2 - l1) * ins);
    return mx;
}

/* distance-type chain (DistanceBase / CachedDistanceBase, distance.hpp:52-76, 120-133,
 * 240-262, 304-317); dist(c) is the metric's _distance under cutoff c */
template <typename DistFn>
void chain_dist(int op, u64 M, DistFn dist, u64 ci, double cf, i64* oi, double* of)
{
    auto ndist = [&](double c) {
        u64 cd = (u64)std::ceil((double)M * c);
        u64 d = dist(cd);
        double nd = M != 0 ? (double)d / (double)M : 0.0;
        return nd <= c ? nd : 1.0;
    };
    switch (op) {
    case RFO_DISTANCE: *oi = (i64)dist(ci); break;
    case RFO_SIMILARITY:
        if (ci > M) *oi = 0;
        else {
            u64 s = M - dist(M - ci);
            *oi = s >= ci ? (i64)s : 0;
        }
        break;
    case RFO_NORM_DISTANCE: *of = ndist(cf); break;
    default: {
        double nd = ndist(norm_sim_to_norm_dist(cf));
        double ns = 1.0 - nd;
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

/* similarity-type chain over integers (SimilarityBase / CachedSimilarityBase, distance.hpp:177-203,
 * 359-369); sim(c) is _similarity under cutoff c */
template <typename SimFn>
void chain_sim(int op, u64 M, SimFn sim, u64 ci, double cf, i64* oi, double* of)
{
    auto dist = [&](u64 c) -> u64 {
        u64 cs = M >= c ? M - c : 0;
        u64 d = M - sim(cs);
        return d <= c ? d : c + 1;
    };
    auto ndist = [&](double c) {
        u64 cd = (u64)std::ceil((double)M * c);
        u64 d = dist(cd);
        double nd = M != 0 ? (double)d / (double)M : 0.0;
        return nd <= c ? nd : 1.0;
    };
    switch (op) {
    case RFO_DISTANCE: *oi = (i64)dist(ci); break;
    case RFO_SIMILARITY: *oi = (i64)sim(ci); break;
    case RFO_NORM_DISTANCE: *of = ndist(cf); break;
    default: {
        double nd = ndist(norm_sim_to_norm_dist(cf));
        double ns = 1.0 - nd;
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

/* similarity-type chain over doubles with maximum 1.0 (Jaro / Jaro-Winkler) */
template <typename SimFn>
void chain_fsim(int op, SimFn sim, double cf, double* of)
{
    auto dist = [&](double c) -> double {
        double cs = 1.0 >= c ? 1.0 - c : 0.0;
        double d = 1.0 - sim(cs);
        return d <= c ? d : 1.0;
    };
    auto ndist = [&](double c) {
        double cd = std::ceil(1.0 * c);
        double nd = dist(cd) / 1.0;
        return nd <= c ? nd : 1.0;
    };
    switch (op) {
    case RFO_DISTANCE: *of = dist(cf); break;
    case RFO_SIMILARITY: *of = sim(cf); break;
    case RFO_NORM_DISTANCE: *of = ndist(cf); break;
    default: {
        double nd = ndist(norm_sim_to_norm_dist(cf));
        double ns = 1.0 - nd;
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

/* Multi* chains (MultiDistanceBase / MultiSimilarityBase / MultiNormalizedMetricBase,
 * distance.hpp:421-460, 500-512, 552-563): exact values, cutoff applied after */
void chain_multi_dist(int op, u64 M, u64 D, u64 ci, double cf, i64* oi, double* of)
{
    switch (op) {
    case RFO_DISTANCE: *oi = (i64)(D <= ci ? D : ci + 1); break;
    case RFO_SIMILARITY: {
        u64 s = M - D;
        *oi = s >= ci ? (i64)s : 0;
        break;
    }
    case RFO_NORM_DISTANCE: {
        double nd = M != 0 ? (double)D / (double)M : 0.0;
        *of = nd <= cf ? nd : 1.0;
        break;
    }
    default: {
        double nd = M != 0 ? (double)D / (double)M : 0.0;
        nd = nd <= 1.0 ? nd : 1.0;
        double ns = 1.0 - nd;
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

void chain_multi_sim(int op, u64 M, u64 S, u64 ci, double cf, i64* oi, double* of)
{
    switch (op) {
    case RFO_SIMILARITY: *oi = S >= ci ? (i64)S : 0; break;
    case RFO_DISTANCE: {
        u64 d = M - S;
        *oi = (i64)(d <= ci ? d : ci + 1);
        break;
    }
    case RFO_NORM_DISTANCE: {
        u64 d = M - S;
        double nd = M != 0 ? (double)d / (double)M : 0.0;
        *of = nd <= cf ? nd : 1.0;
        break;
    }
    default: {
        u64 d = M - S;
        double nd = M != 0 ? (double)d / (double)M : 0.0;
        nd = nd <= 1.0 ? nd : 1.0;
        double ns = 1.0 - nd;
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

/* sim_at(c) is the Multi scorer's _similarity under cutoff c */
template <typename SimAt>
void chain_multi_fsim(int op, SimAt sim_at, double cf, double* of)
{
    switch (op) {
    case RFO_SIMILARITY: *of = sim_at(cf); break;
    case RFO_DISTANCE: {
        double d = 1.0 - sim_at(0.0);
        *of = d <= cf ? d : 1.0;
        break;
    }
    case RFO_NORM_DISTANCE: {
        double d = 1.0 - sim_at(0.0);
        d = d <= 1.0 ? d : 1.0;
        *of = d <= cf ? d : 1.0;
        break;
    }
    default: {
        double d = 1.0 - sim_at(0.0);
        d = d <= 1.0 ? d : 1.0;
        double ns = 1.0 - d;
        *of = ns >= cf ? ns : 0.0;
    }
    }
}

/* =============================================== exact values with a cached PM */

template <typename S1, typename S2>
u64 lev_weighted_cached(const PM& pm, const S1& s1, const S2& s2, const rfo_params* w, u64 cutoff, u64 hint);

/* generalized Wagner-Fischer (Levenshtein_impl.hpp:85-155), affix stripped */
template <typename S1, typename S2>
u64 lev_generalized(const S1& s1in, const S2& s2in, const rfo_params* w, u64 max)
{
    const u64 ins = (u64)w->insert_cost, del = (u64)w->delete_cost, rep = (u64)w->replace_cost;
    u64 min_edits = s1in.n > s2in.n ? (u64)(s1in.n - s2in.n) * del : (u64)(s2in.n - s1in.n) * ins;
    if (min_edits > max) return max + 1;
    i64 a0 = 0, a1 = s1in.n, b0 = 0, b1 = s2in.n;
    while (a0 < a1 && b0 < b1 && s1in[a0] == s2in[b0]) ++a0, ++b0;
    while (a0 < a1 && b0 < b1 && s1in[a1 - 1] == s2in[b1 - 1]) --a1, --b1;
    const i64 m = a1 - a0;
    std::vector<u64> cache(m + 1);
    for (i64 i = 0; i <= m; ++i) cache[i] = (u64)i * del;
    for (i64 j = b0; j < b1; ++j) {
        u64 temp = cache[0];
        cache[0] += ins;
        for (i64 i = 0; i < m; ++i) {
            if (s1in[a0 + i] != s2in[j]) temp = std::min({cache[i] + del, cache[i + 1] + ins, temp + rep});
            std::swap(cache[i + 1], temp);
        }
    }
    u64 d = cache[m];
    return d <= max ? d : max + 1;
}

/* levenshtein_distance with weights (Levenshtein_impl.hpp:1056-1089; CachedLevenshtein
 * Levenshtein.hpp:445-477 takes the same branches with the cached pattern) */
template <typename S1, typename S2>
u64 lev_weighted_cached(const PM& pm, const S1& s1, const S2& s2, const rfo_params* w, u64 cutoff, u64 hint)
{
    const u64 ins = (u64)w->insert_cost, del = (u64)w->delete_cost, rep = (u64)w->replace_cost;
    if (ins == del) {
        if (ins == 0) return 0;
        if (ins == rep) {
            u64 d = lev_uniform_cached(pm, s1, s2, ceil_div_u(cutoff, ins), ceil_div_u(hint, ins)) * ins;
            return d <= cutoff ? d : cutoff + 1;
        }
        if (rep >= ins + del) {
            u64 nc = ceil_div_u(cutoff, ins);
            u64 M = (u64)(s1.n + s2.n);
            u64 lcs_cut = (M / 2 >= nc) ? M / 2 - nc : 0;
            u64 l = lcs_cached(pm, s1, s2, lcs_cut);
            u64 di = M - 2 * l;
            di = di <= nc ? di : nc + 1;
            u64 d = di * ins;
            return d <= cutoff ? d : cutoff + 1;
        }
    }
    return lev_generalized(s1, s2, w, cutoff);
}

/* Indel::_distance via the cached LCS (Indel.hpp:170-179) */
template <typename S1, typename S2>
u64 indel_cached(const PM& pm, const S1& s1, const S2& s2, u64 cutoff)
{
    u64 M = (u64)(s1.n + s2.n);
    u64 lcs_cut = (M / 2 >= cutoff) ? M / 2 - cutoff : 0;
    u64 l = lcs_cached(pm, s1, s2, lcs_cut);
    u64 d = M - 2 * l;
    return d <= cutoff ? d : cutoff + 1;
}

/* one scorer call with a prebuilt pattern of s1 */
template <typename S1, typename S2>
int score_with_pm(int metric, int op, int form, const PM& pm, const S1& s1, const S2& s2, const rfo_params* p,
                  u64 ci, double cf, i64* oi, double* of)
{
    const u64 l1 = (u64)s1.n, l2 = (u64)s2.n;
    const u64 HINT = std::numeric_limits<u64>::max();
    if (form == RFO_FORM_MULTI) {
        switch (metric) {
        case RFO_LEVENSHTEIN: {
            if (p->delete_cost != 1 || p->insert_cost != 1 || p->replace_cost > 2) return -1;
            u64 D = lev_uniform_cached(pm, s1, s2, HINT, HINT);
            chain_multi_dist(op, lev_maximum(l1, l2, p), D, ci, cf, oi, of);
            return 0;
        }
        case RFO_OSA: {
            u64 D = osa_cached(pm, s1, s2, HINT);
            chain_multi_dist(op, std::max(l1, l2), D, ci, cf, oi, of);
            return 0;
        }
        case RFO_INDEL: {
            u64 L = s1.n ? (u64)lcs_full(pm, s2) : 0;
            chain_multi_dist(op, l1 + l2, l1 + l2 - 2 * L, ci, cf, oi, of);
            return 0;
        }
        case RFO_LCSSEQ: {
            u64 L = s1.n ? (u64)lcs_full(pm, s2) : 0;
            chain_multi_sim(op, std::max(l1, l2), L, ci, cf, oi, of);
            return 0;
        }
        case RFO_RATIO: {
            if (op != RFO_SIMILARITY) return -1;
            u64 L = s1.n ? (u64)lcs_full(pm, s2) : 0;
            double r;
            chain_multi_dist(RFO_NORM_SIMILARITY, l1 + l2, l1 + l2 - 2 * L, 0, cf / 100.0, oi, &r);
            *of = r * 100.0;
            return 0;
        }
        case RFO_TOKEN_SORT_RATIO:
        case RFO_QRATIO: {
            if (op != RFO_SIMILARITY) return -1;
            *of = token_multi(metric, s1, s2, cf);
            return 0;
        }
        case RFO_JARO:
        case RFO_JARO_WINKLER: {
            i64 C, T;
            jaro_counts_pm(pm, s1, s2, &C, &T);
            i64 prefix = common_prefix4(s1, s2);
            auto sim_at = [&](double c) {
                if (metric == RFO_JARO) return multi_jaro_from_counts(s1.n, s2.n, C, T, c);
                double js = multi_jaro_from_counts(s1.n, s2.n, C, T, std::min(0.7, c));
                return multi_jw(js, prefix, p->prefix_weight, c);
            };
            chain_multi_fsim(op, sim_at, cf, of);
            return 0;
        }
        }
        return -1;
    }

    switch (metric) {
    case RFO_LEVENSHTEIN: {
        auto dist = [&](u64 c) { return lev_weighted_cached(pm, s1, s2, p, c, HINT); };
        chain_dist(op, lev_maximum(l1, l2, p), dist, ci, cf, oi, of);
        return 0;
    }
    case RFO_INDEL: {
        auto dist = [&](u64 c) { return indel_cached(pm, s1, s2, c); };
        chain_dist(op, l1 + l2, dist, ci, cf, oi, of);
        return 0;
    }
    case RFO_OSA: {
        auto dist = [&](u64 c) { return osa_cached(pm, s1, s2, c); };
        chain_dist(op, std::max(l1, l2), dist, ci, cf, oi, of);
        return 0;
    }
    case RFO_LCSSEQ: {
        auto sim = [&](u64 c) { return lcs_cached(pm, s1, s2, c); };
        chain_sim(op, std::max(l1, l2), sim, ci, cf, oi, of);
        return 0;
    }
    case RFO_PARTIAL_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        *of = partial_ratio_score(s1, s2, cf);
        return 0;
    }
    case RFO_TOKEN_SORT_RATIO:
    case RFO_PARTIAL_TOKEN_SORT_RATIO:
    case RFO_QRATIO: {
        if (op != RFO_SIMILARITY) return -1;
        *of = token_scorer(metric, s1, s2, cf);
        return 0;
    }
    case RFO_TOKEN_SET_RATIO:
    case RFO_PARTIAL_TOKEN_SET_RATIO:
    case RFO_TOKEN_RATIO:
    case RFO_PARTIAL_TOKEN_RATIO:
    case RFO_WRATIO: {
        if (op != RFO_SIMILARITY) return -1;
        *of = token_set_family(metric, s1, s2, cf);
        return 0;
    }
    case RFO_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        auto dist = [&](u64 c) { return indel_cached(pm, s1, s2, c); };
        double r;
        chain_dist(RFO_NORM_SIMILARITY, l1 + l2, dist, 0, cf / 100.0, oi, &r);
        *of = r * 100.0;
        return 0;
    }
    case RFO_JARO:
    case RFO_JARO_WINKLER: {
        i64 C = -1, T = 0;
        auto jaro = [&](double c) {
            if (c > 1.0) return 0.0;
            if (!s1.n && !s2.n) return 1.0;
            if (!jaro_length_filter(s1.n, s2.n, c)) return 0.0;
            if (C < 0) jaro_counts_pm(pm, s1, s2, &C, &T);
            return jaro_from_counts(s1.n, s2.n, C, T, c);
        };
        if (metric == RFO_JARO) {
            chain_fsim(op, jaro, cf, of);
        }
        else {
            i64 prefix = common_prefix4(s1, s2);
            auto jw = [&](double c) { return jw_chain(prefix, p->prefix_weight, c, jaro); };
            chain_fsim(op, jw, cf, of);
        }
        return 0;
    }
    }
    return -1;
}

/* ------------------------------------------------------------- partial_ratio
 * fuzz::partial_ratio / CachedPartialRatio::similarity (fuzz_impl.hpp:49-293): the best
 * fuzz::ratio of the shorter string against every window of its length in the longer
 * one (searched by bisection with a distance bound, fuzz_impl.hpp:82-149), and against
 * the shorter prefixes and suffixes of the longer string whose edge unit occurs in the
 * shorter (fuzz_impl.hpp:151-175); equal lengths also try the other direction
 * (fuzz_impl.hpp:215-224). */

/* CachedRatio::similarity (fuzz_impl.hpp:43-47) of needle against sub */
template <typename S1, typename S2>
double ratio_with_pm(const PM& pm, const S1& needle, const S2& sub, double cutoff)
{
    auto dist = [&](u64 c) { return indel_cached(pm, needle, sub, c); };
    double r = 0;
    i64 oi = 0;
    chain_dist(RFO_NORM_SIMILARITY, (u64)needle.n + (u64)sub.n, dist, 0, cutoff / 100.0, &oi, &r);
    return r * 100.0;
}

template <typename S1, typename S2>
bool char_in(const S1& s, u64 c)
{
    for (i64 i = 0; i < s.n; ++i)
        if (s[i] == c) return true;
    return false;
}

/* partial_ratio_impl: s1 no longer than s2, both non-empty */
template <typename S1, typename S2>
double partial_impl(const S1& s1, const S2& s2, double cutoff)
{
    PM pm;
    pm.build(s1);
    const i64 len1 = s1.n, len2 = s2.n;
    double res = 0.0;
    if (len2 > len1) {
        const u64 maximum = (u64)len1 * 2;
        const double ncs = norm_sim_to_norm_dist(cutoff / 100);
        u64 cutoff_dist = (u64)std::ceil((double)maximum * ncs);
        u64 best = std::numeric_limits<u64>::max();
        const u64 NONE = std::numeric_limits<u64>::max();
        std::vector<u64> scores((size_t)(len2 - len1), NONE);
        std::vector<std::pair<i64, i64>> windows = {{0, len2 - len1 - 1}}, next;
        auto eval = [&](i64 pos) -> bool { /* true: a perfect window */
            if (scores[(size_t)pos] != NONE) return false;
            S2 sub{s2.p + pos, len1};
            scores[(size_t)pos] = indel_cached(pm, s1, sub, NONE);
            if (scores[(size_t)pos] < cutoff_dist) {
                cutoff_dist = best = scores[(size_t)pos];
                if (best == 0) return true;
            }
            return false;
        };
        while (!windows.empty()) {
            for (const auto& w : windows) {
                if (eval(w.first)) return 100.0;
                if (eval(w.second)) return 100.0;
                const u64 cell_diff = (u64)(w.second - w.first);
                if (cell_diff == 1) continue;
                const u64 a = scores[(size_t)w.first], b = scores[(size_t)w.second];
                const u64 known = a > b ? a - b : b - a;
                const u64 max_imp = (cell_diff - known / 2) / 2 * 2;
                const i64 min_score = (i64)std::min(a, b) - (i64)max_imp;
                if (min_score < (i64)cutoff_dist) {
                    const i64 center = (i64)(cell_diff / 2);
                    next.emplace_back(w.first, w.first + center);
                    next.emplace_back(w.first + center, w.second);
                }
            }
            std::swap(windows, next);
            next.clear();
        }
        double score = 1.0 - (double)best / (double)maximum;
        score *= 100;
        if (score >= cutoff) cutoff = res = score;
    }
    for (i64 i = 1; i < len1; ++i) {
        S2 sub{s2.p, i};
        if (!char_in<S1, S2>(s1, sub[i - 1])) continue;
        const double r = ratio_with_pm(pm, s1, sub, cutoff);
        if (r > res) {
            cutoff = res = r;
            if (res == 100.0) return res;
        }
    }
    for (i64 i = len2 - len1; i < len2; ++i) {
        S2 sub{s2.p + i, len2 - i};
        if (!char_in<S1, S2>(s1, sub[0])) continue;
        const double r = ratio_with_pm(pm, s1, sub, cutoff);
        if (r > res) {
            cutoff = res = r;
            if (res == 100.0) return res;
        }
    }
    return res;
}

/* partial_ratio_alignment(...).score (fuzz_impl.hpp:194-227) */
template <typename S1, typename S2>
double partial_ratio_score(const S1& s1, const S2& s2, double cutoff)
{
    if (s1.n > s2.n) return partial_ratio_score(s2, s1, cutoff);
    if (cutoff > 100) return 0.0;
    if (!s1.n || !s2.n) return (double)(s1.n == s2.n) * 100.0;
    const double score = partial_impl(s1, s2, cutoff);
    if (score != 100 && s1.n == s2.n) {
        cutoff = std::max(cutoff, score);
        const double score2 = partial_impl(s2, s1, cutoff);
        if (score2 > score) return score2;
    }
    return score;
}

/* ------------------------------------------------ token_sort_ratio, QRatio
 * token_sort_ratio / partial_token_sort_ratio (fuzz_impl.hpp:294-360): ratio /
 * partial_ratio of both strings after sorted_split(...).join() (common_impl.hpp:162-180,
 * SplittedSentenceView.hpp:71-85): split on whitespace, drop empty tokens, sort the
 * tokens lexicographically by code unit, join with U+0020.  Whitespace follows the
 * code-unit size (common_impl.hpp:85-152): one-byte units know the ASCII set only.
 * QRatio (fuzz_impl.hpp:887-931): 0 when either string is empty, else ratio. */
bool unit_is_space(u64 c, bool one_byte)
{
    switch (c) {
    case 0x09: case 0x0A: case 0x0B: case 0x0C: case 0x0D: case 0x1C: case 0x1D: case 0x1E: case 0x1F:
    case 0x20: return true;
    }
    if (one_byte) return false;
    switch (c) {
    case 0x85: case 0xA0: case 0x1680: case 0x2000: case 0x2001: case 0x2002: case 0x2003: case 0x2004:
    case 0x2005: case 0x2006: case 0x2007: case 0x2008: case 0x2009: case 0x200A: case 0x2028: case 0x2029:
    case 0x202F: case 0x205F: case 0x3000: return true;
    }
    return false;
}

using Tokens = std::vector<std::vector<u64>>;

/* sorted_split (common_impl.hpp:162-180): the tokens, sorted */
template <typename S>
Tokens sorted_tokens(const S& s, bool one_byte)
{
    Tokens toks;
    std::vector<u64> cur;
    for (i64 i = 0; i <= s.n; ++i) {
        if (i == s.n || unit_is_space(s[i], one_byte)) {
            if (!cur.empty()) toks.push_back(cur);
            cur.clear();
        }
        else cur.push_back(s[i]);
    }
    std::sort(toks.begin(), toks.end());
    return toks;
}

/* SplittedSentenceView::join (SplittedSentenceView.hpp:71-85) */
std::vector<u64> join_tokens(const Tokens& toks)
{
    std::vector<u64> out;
    for (size_t k = 0; k < toks.size(); ++k) {
        if (k) out.push_back(0x20);
        out.insert(out.end(), toks[k].begin(), toks[k].end());
    }
    return out;
}

template <typename S>
std::vector<u64> sorted_join(const S& s, bool one_byte)
{
    return join_tokens(sorted_tokens(s, one_byte));
}

/* fuzz::ratio (fuzz_impl.hpp:28-32) */
template <typename S1, typename S2>
double ratio_plain(const S1& a, const S2& b, double cutoff)
{
    PM pm;
    pm.build(a);
    return ratio_with_pm(pm, a, b, cutoff);
}

template <typename S1, typename S2>
double token_scorer(int metric, const S1& s1, const S2& s2, double cutoff)
{
    if (metric == RFO_QRATIO) {
        if (!s1.n || !s2.n) return 0.0;
        return ratio_plain(s1, s2, cutoff);
    }
    if (cutoff > 100) return 0.0;
    const std::vector<u64> a = sorted_join(s1, sizeof(s1.p[0]) == 1), b = sorted_join(s2, sizeof(s2.p[0]) == 1);
    const Str<u64> sa{a.data(), (i64)a.size()}, sb{b.data(), (i64)b.size()};
    if (metric == RFO_TOKEN_SORT_RATIO) return ratio_plain(sa, sb, cutoff);
    return partial_ratio_score(sa, sb, cutoff);
}

/* MultiRatio's chain for one inserted string (fuzz.hpp:50-95 over MultiIndel) */
template <typename S1, typename S2>
double multi_ratio(const S1& a, const S2& b, double cutoff)
{
    PM pm;
    pm.build(a);
    const u64 L = a.n ? (u64)lcs_full(pm, b) : 0, M = (u64)(a.n + b.n);
    double r;
    chain_multi_dist(RFO_NORM_SIMILARITY, M, M - 2 * L, 0, cutoff / 100.0, nullptr, &r);
    return r * 100.0;
}

/* MultiTokenSortRatio (fuzz.hpp:236-278): MultiRatio over the sorted-split joins;
 * MultiQRatio (fuzz.hpp:719-774): 0 when either string is empty, else MultiRatio */
template <typename S1, typename S2>
double token_multi(int metric, const S1& s1, const S2& s2, double cutoff)
{
    if (metric == RFO_QRATIO) {
        if (!s1.n || !s2.n) return 0.0;
        return multi_ratio(s1, s2, cutoff);
    }
    const std::vector<u64> a = sorted_join(s1, sizeof(s1.p[0]) == 1), b = sorted_join(s2, sizeof(s2.p[0]) == 1);
    return multi_ratio(Str<u64>{a.data(), (i64)a.size()}, Str<u64>{b.data(), (i64)b.size()}, cutoff);
}

/* ------------------------------------------------ token_set_ratio, token_ratio, WRatio
 * set_decomposition (common_impl.hpp:11-35): both sorted token lists lose adjacent
 * duplicates, then each token of a is looked up in what is left of b: found tokens form
 * the intersection (in a's order) and leave b, the others form diff_ab; the rest of b
 * is diff_ba. */
struct Decomp {
    Tokens ab, ba, sect;
};

Decomp decompose(Tokens a, Tokens b)
{
    a.erase(std::unique(a.begin(), a.end()), a.end());
    b.erase(std::unique(b.begin(), b.end()), b.end());
    Decomp d;
    d.ba = b;
    for (const auto& t : a) {
        auto it = std::find(d.ba.begin(), d.ba.end(), t);
        if (it != d.ba.end()) {
            d.ba.erase(it);
            d.sect.push_back(t);
        }
        else d.ab.push_back(t);
    }
    return d;
}

/* SplittedSentenceView::size (SplittedSentenceView.hpp:56-69): the joined length */
u64 joined_len(const Tokens& t)
{
    if (t.empty()) return 0;
    u64 n = t.size() - 1;
    for (const auto& x : t) n += x.size();
    return n;
}

/* norm_distance, score_cutoff_to_distance (fuzz_impl.hpp:55-66) */
double norm_distance_pct(u64 dist, u64 lensum, double cutoff)
{
    const double score = lensum > 0 ? 100.0 - 100.0 * (double)dist / (double)lensum : 100.0;
    return score >= cutoff ? score : 0;
}

u64 cutoff_to_distance(double cutoff, u64 lensum)
{
    return (u64)std::ceil((double)lensum * (1.0 - cutoff / 100));
}

Str<u64> view(const std::vector<u64>& v) { return Str<u64>{v.data(), (i64)v.size()}; }

/* indel_distance(a, b, cutoff): exact when <= cutoff, else cutoff + 1 */
u64 indel_dist(const std::vector<u64>& a, const std::vector<u64>& b, u64 cutoff)
{
    PM pm;
    pm.build(view(a));
    return indel_cached(pm, view(a), view(b), cutoff);
}

/* the common part of token_set_ratio (fuzz_impl.hpp:372-420) and token_ratio
 * (fuzz_impl.hpp:518-564); with_sorted adds ratio(tokens_a.join(), tokens_b.join()) */
double token_set_tail(const Tokens& ta, const Tokens& tb, double cutoff, bool with_sorted)
{
    const Decomp d = decompose(ta, tb);
    if (!d.sect.empty() && (d.ab.empty() || d.ba.empty())) return 100;
    const std::vector<u64> ab = join_tokens(d.ab), ba = join_tokens(d.ba);
    const u64 ab_len = ab.size(), ba_len = ba.size(), sect_len = joined_len(d.sect);
    double result = 0;
    if (with_sorted) {
        const std::vector<u64> ja = join_tokens(ta), jb = join_tokens(tb);
        result = ratio_plain(view(ja), view(jb), cutoff);
    }
    const u64 sect_ab_len = sect_len + (sect_len != 0) + ab_len, sect_ba_len = sect_len + (sect_len != 0) + ba_len;
    const u64 cd = cutoff_to_distance(cutoff, sect_ab_len + sect_ba_len);
    const u64 dist = indel_dist(ab, ba, cd);
    if (dist <= cd) {
        const double nd = norm_distance_pct(dist, sect_ab_len + sect_ba_len, cutoff);
        result = with_sorted ? std::max(result, nd) : nd;
    }
    if (!sect_len) return result;
    const double r_ab = norm_distance_pct((sect_len != 0) + ab_len, sect_len + sect_ab_len, cutoff);
    const double r_ba = norm_distance_pct((sect_len != 0) + ba_len, sect_len + sect_ba_len, cutoff);
    return std::max({result, r_ab, r_ba});
}

/* partial_token_ratio (fuzz_impl.hpp:704-731) */
double partial_token_ratio_toks(const Tokens& ta, const Tokens& tb, double cutoff)
{
    if (cutoff > 100) return 0;
    const Decomp d = decompose(ta, tb);
    if (!d.sect.empty()) return 100;
    const std::vector<u64> ja = join_tokens(ta), jb = join_tokens(tb);
    const double result = partial_ratio_score(view(ja), view(jb), cutoff);
    if (ta.size() == d.ab.size() && tb.size() == d.ba.size()) return result;
    cutoff = std::max(cutoff, result);
    const std::vector<u64> ab = join_tokens(d.ab), ba = join_tokens(d.ba);
    return std::max(result, partial_ratio_score(view(ab), view(ba), cutoff));
}

/* token_ratio (fuzz_impl.hpp:518-564) */
double token_ratio_toks(const Tokens& ta, const Tokens& tb, double cutoff)
{
    if (cutoff > 100) return 0;
    return token_set_tail(ta, tb, cutoff, true);
}

/* token_set_ratio, partial_token_set_ratio, token_ratio, partial_token_ratio, WRatio
 * (fuzz_impl.hpp:373-889); the Cached forms give the same values */
template <typename S1, typename S2>
double token_set_family(int metric, const S1& s1, const S2& s2, double cutoff)
{
    if (cutoff > 100) return 0;
    const bool ob1 = sizeof(s1.p[0]) == 1, ob2 = sizeof(s2.p[0]) == 1;
    switch (metric) {
    case RFO_TOKEN_SET_RATIO: {
        const Tokens ta = sorted_tokens(s1, ob1), tb = sorted_tokens(s2, ob2);
        if (ta.empty() || tb.empty()) return 0;
        return token_set_tail(ta, tb, cutoff, false);
    }
    case RFO_PARTIAL_TOKEN_SET_RATIO: {
        const Tokens ta = sorted_tokens(s1, ob1), tb = sorted_tokens(s2, ob2);
        if (ta.empty() || tb.empty()) return 0;
        const Decomp d = decompose(ta, tb);
        if (!d.sect.empty()) return 100;
        const std::vector<u64> ab = join_tokens(d.ab), ba = join_tokens(d.ba);
        return partial_ratio_score(view(ab), view(ba), cutoff);
    }
    case RFO_TOKEN_RATIO: return token_ratio_toks(sorted_tokens(s1, ob1), sorted_tokens(s2, ob2), cutoff);
    case RFO_PARTIAL_TOKEN_RATIO:
        return partial_token_ratio_toks(sorted_tokens(s1, ob1), sorted_tokens(s2, ob2), cutoff);
    default: break;
    }
    /* WRatio (fuzz_impl.hpp:789-822) */
    const double UNBASE_SCALE = 0.95;
    const i64 len1 = s1.n, len2 = s2.n;
    if (!len1 || !len2) return 0;
    const double len_ratio = len1 > len2 ? (double)len1 / (double)len2 : (double)len2 / (double)len1;
    double end_ratio = ratio_plain(s1, s2, cutoff);
    if (len_ratio < 1.5) {
        cutoff = std::max(cutoff, end_ratio) / UNBASE_SCALE;
        return std::max(end_ratio, token_ratio_toks(sorted_tokens(s1, ob1), sorted_tokens(s2, ob2), cutoff) *
                                       UNBASE_SCALE);
    }
    const double PARTIAL_SCALE = len_ratio <= 8.0 ? 0.9 : 0.6;
    cutoff = std::max(cutoff, end_ratio) / PARTIAL_SCALE;
    end_ratio = std::max(end_ratio, partial_ratio_score(s1, s2, cutoff) * PARTIAL_SCALE);
    cutoff = std::max(cutoff, end_ratio) / UNBASE_SCALE;
    return std::max(end_ratio, partial_token_ratio_toks(sorted_tokens(s1, ob1), sorted_tokens(s2, ob2), cutoff) *
                                   UNBASE_SCALE * PARTIAL_SCALE);
}

template <typename T>
void store(void* out, int dtype, i64 idx, i64 vi, double vf, bool is_int)
{
    (void)sizeof(T);
    if (dtype == 0) ((int32_t*)out)[idx] = (int32_t)vi;
    else if (dtype == 1) ((int64_t*)out)[idx] = vi;
    else ((double*)out)[idx] = is_int ? (double)vi : vf;
}

bool result_is_int(int metric, int op)
{
    if (metric == RFO_JARO || metric == RFO_JARO_WINKLER || metric >= RFO_RATIO) return false;
    return op == RFO_DISTANCE || op == RFO_SIMILARITY;
}

} // namespace

/* ====================================================================== C ABI */

/* ------------------------------------------------ editops
 * The reference recovers an alignment from bit matrices recorded row by row over s2
 * (LCSseq_impl.hpp:437-529 recover_alignment / lcs_matrix; Levenshtein_impl.hpp:956-1021
 * recover_alignment, 1023-1045 levenshtein_align): after the common prefix and suffix are
 * removed, bit c of row r says, for the first r + 1 units of s2, whether the table's value
 * grows from s1 prefix c to c + 1 (Levenshtein: VP = +1, VN = -1; LCS: S = the LCS does
 * NOT grow).  This restatement builds those bits from the full DP tables (not from bit
 * vectors) and walks back from the end as the reference does.  The reference's banded
 * Levenshtein matrices (a score_hint, or a source longer than 64 units) gave the same
 * walk as the full tables on every pair checked against it.  Long Levenshtein pairs go
 * through the reference's Hirschberg recursion (Levenshtein_impl.hpp:1090-1257): split s2
 * in half, take the first s1 position minimising left + right distance, recurse. */
using Units = std::vector<u64>;

/* one segment's alignment from its DP table, written to out[pos, pos + dist) */
void align_dp(bool lev, const u64* A, i64 m, const u64* B, i64 n, i64 src_pos, i64 dest_pos, i64 pos,
              std::vector<rfo_editop>* out)
{
    std::vector<i64> T((size_t)(m + 1) * (n + 1));
    auto at = [&](i64 i, i64 j) -> i64& { return T[(size_t)i * (n + 1) + j]; };
    for (i64 i = 0; i <= m; ++i)
        for (i64 j = 0; j <= n; ++j) {
            if (lev) {
                if (!i || !j) at(i, j) = i + j;
                else at(i, j) = std::min({at(i - 1, j) + 1, at(i, j - 1) + 1, at(i - 1, j - 1) + (A[i - 1] != B[j - 1])});
            }
            else {
                if (!i || !j) at(i, j) = 0;
                else at(i, j) = A[i - 1] == B[j - 1] ? at(i - 1, j - 1) + 1 : std::max(at(i - 1, j), at(i, j - 1));
            }
        }
    /* bit col of row r (s2 prefix r + 1) */
    auto vp = [&](i64 r, i64 col) { return at(col + 1, r + 1) - at(col, r + 1) == 1; };
    auto vn = [&](i64 r, i64 col) { return at(col + 1, r + 1) - at(col, r + 1) == -1; };
    auto sbit = [&](i64 r, i64 col) { return at(col + 1, r + 1) - at(col, r + 1) == 0; };
    i64 dist = lev ? at(m, n) : m + n - 2 * at(m, n);
    if ((i64)out->size() < pos + dist) out->resize((size_t)(pos + dist), rfo_editop{0, 0, 0, 0});
    auto put = [&](int type, i64 col, i64 row) {
        --dist;
        (*out)[(size_t)(pos + dist)] = rfo_editop{type, 0, col + src_pos, row + dest_pos};
    };
    i64 col = m, row = n;
    if (dist == 0) return;
    while (row && col) {
        if (lev ? vp(row - 1, col - 1) : sbit(row - 1, col - 1)) {
            --col;
            put(3, col, row);
        }
        else {
            --row;
            if (row && (lev ? vn(row - 1, col - 1) : !sbit(row - 1, col - 1)))
                put(2, col, row);
            else {
                --col;
                if (lev && A[col] != B[row]) put(1, col, row);
            }
        }
    }
    while (col) {
        --col;
        put(3, col, row);
    }
    while (row) {
        --row;
        put(2, col, row);
    }
}

/* the Levenshtein DP row of A[0, m) against B[0, n): row[i] = D(A[0, i), B[0, n)) */
std::vector<i64> lev_row(const u64* A, i64 m, const u64* B, i64 n)
{
    std::vector<i64> prev((size_t)m + 1), cur((size_t)m + 1);
    for (i64 i = 0; i <= m; ++i) prev[i] = i;
    for (i64 j = 1; j <= n; ++j) {
        cur[0] = j;
        for (i64 i = 1; i <= m; ++i)
            cur[i] = std::min({prev[i] + 1, cur[i - 1] + 1, prev[i - 1] + (A[i - 1] != B[j - 1])});
        std::swap(prev, cur);
    }
    return prev;
}

/* levenshtein_align_hirschberg (Levenshtein_impl.hpp:1184-1213) on A[0, m), B[0, n) */
void align_hirschberg(const u64* A, i64 m, const u64* B, i64 n, i64 src_pos, i64 dest_pos, i64 pos, u64 max,
                      std::vector<rfo_editop>* out)
{
    i64 pre = 0;
    while (pre < m && pre < n && A[pre] == B[pre]) ++pre;
    i64 suf = 0;
    while (suf < m - pre && suf < n - pre && A[m - 1 - suf] == B[n - 1 - suf]) ++suf;
    A += pre;
    B += pre;
    m -= pre + suf;
    n -= pre + suf;
    src_pos += pre;
    dest_pos += pre;
    max = std::min<u64>(max, (u64)std::max(m, n));
    const u64 full_band = std::min<u64>((u64)m, 2 * max + 1);
    const u64 matrix_size = 2 * full_band * (u64)n / 8;
    if (matrix_size < 1024 * 1024 || m < 65 || n < 10) {
        align_dp(true, A, m, B, n, src_pos, dest_pos, pos, out);
        return;
    }
    /* find_hirschberg_pos (Levenshtein_impl.hpp:1096-1180) */
    const i64 s2_mid = n / 2;
    const std::vector<i64> left = lev_row(A, m, B, s2_mid);
    Units ra(A, A + m), rb(B + s2_mid, B + n);
    std::reverse(ra.begin(), ra.end());
    std::reverse(rb.begin(), rb.end());
    const std::vector<i64> right = lev_row(ra.data(), m, rb.data(), n - s2_mid);
    i64 best = std::numeric_limits<i64>::max(), s1_mid = 0, ls = 0, rs = 0;
    for (i64 i = 0; i <= m; ++i)
        if (left[i] + right[m - i] < best) {
            best = left[i] + right[m - i];
            s1_mid = i;
            ls = left[i];
            rs = right[m - i];
        }
    align_hirschberg(A, s1_mid, B, s2_mid, src_pos, dest_pos, pos, (u64)ls, out);
    align_hirschberg(A + s1_mid, m - s1_mid, B + s2_mid, n - s2_mid, src_pos + s1_mid, dest_pos + s2_mid, pos + ls,
                     (u64)rs, out);
}

template <typename S1, typename S2>
int editops_impl(int metric, const S1& a0, const S2& b0, u64 hint, std::vector<rfo_editop>* out)
{
    Units A((size_t)a0.n), B((size_t)b0.n);
    for (i64 i = 0; i < a0.n; ++i) A[i] = (u64)a0[i];
    for (i64 j = 0; j < b0.n; ++j) B[j] = (u64)b0[j];
    out->clear();
    if (metric != RFO_LEVENSHTEIN) { /* lcs_seq_editops: common affix, then one table */
        i64 pre = 0;
        while (pre < a0.n && pre < b0.n && A[pre] == B[pre]) ++pre;
        i64 suf = 0;
        while (suf < a0.n - pre && suf < b0.n - pre && A[a0.n - 1 - suf] == B[b0.n - 1 - suf]) ++suf;
        align_dp(false, A.data() + pre, a0.n - pre - suf, B.data() + pre, b0.n - pre - suf, pre, pre, 0, out);
        return 0;
    }
    /* levenshtein_editops (Levenshtein_impl.hpp:1234-1257): the exact distance becomes the
     * band when a small hint makes that worth it */
    if (hint < 31) hint = 31;
    u64 cutoff = (u64)std::max(a0.n, b0.n);
    if (std::numeric_limits<u64>::max() / 2 > hint && 2 * hint < cutoff)
        cutoff = (u64)lev_row(A.data(), a0.n, B.data(), b0.n)[(size_t)a0.n];
    align_hirschberg(A.data(), a0.n, B.data(), b0.n, 0, 0, 0, cutoff, out);
    return 0;
}

extern "C" {

int64_t rfo_levenshtein_exact(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb, int64_t ins,
                              int64_t del, int64_t rep)
{
    rfo_params p{ins, del, rep, 0.1};
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> i64 {
        PM pm;
        pm.build(s1);
        const u64 H = std::numeric_limits<u64>::max() / 4;
        return (i64)lev_weighted_cached(pm, s1, s2, &p, H, H);
    });
}

int64_t rfo_lcs_exact(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb)
{
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> i64 {
        if (!s1.n) return 0;
        PM pm;
        pm.build(s1);
        return lcs_full(pm, s2);
    });
}

int64_t rfo_osa_exact(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb)
{
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> i64 {
        PM pm;
        pm.build(s1);
        return (i64)osa_cached(pm, s1, s2, std::numeric_limits<u64>::max() / 4);
    });
}

void rfo_jaro_counts(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb, int64_t* common,
                     int64_t* transp)
{
    with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> int {
        PM pm;
        pm.build(s1);
        jaro_counts_pm(pm, s1, s2, common, transp);
        return 0;
    });
}

/* rapidfuzz_reference/Levenshtein.hpp: full weighted DP matrix */
int64_t rfo_dp_levenshtein(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb, int64_t ins,
                           int64_t del, int64_t rep)
{
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> i64 {
        std::vector<i64> prev(s1.n + 1), cur(s1.n + 1);
        for (i64 i = 0; i <= s1.n; ++i) prev[i] = i * del;
        for (i64 j = 1; j <= s2.n; ++j) {
            cur[0] = j * ins;
            for (i64 i = 1; i <= s1.n; ++i) {
                i64 sub = prev[i - 1] + (s1[i - 1] == s2[j - 1] ? 0 : rep);
                cur[i] = std::min({prev[i] + ins, cur[i - 1] + del, sub});
            }
            std::swap(prev, cur);
        }
        return prev[s1.n];
    });
}

/* rapidfuzz_reference/LCSseq.hpp */
int64_t rfo_dp_lcs(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb)
{
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> i64 {
        std::vector<i64> prev(s2.n + 1, 0), cur(s2.n + 1, 0);
        for (i64 i = 1; i <= s1.n; ++i) {
            for (i64 j = 1; j <= s2.n; ++j)
                cur[j] = s1[i - 1] == s2[j - 1] ? prev[j - 1] + 1 : std::max(prev[j], cur[j - 1]);
            std::swap(prev, cur);
        }
        return prev[s2.n];
    });
}

/* rapidfuzz_reference/OSA.hpp:13-52 */
int64_t rfo_dp_osa(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb)
{
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> i64 {
        const i64 n1 = s1.n, n2 = s2.n;
        std::vector<i64> M((n1 + 1) * (n2 + 1));
        auto at = [&](i64 i, i64 j) -> i64& { return M[i * (n2 + 1) + j]; };
        for (i64 i = 0; i <= n1; ++i) at(i, 0) = i;
        for (i64 j = 0; j <= n2; ++j) at(0, j) = j;
        for (i64 i = 0; i < n1; ++i)
            for (i64 j = 0; j < n2; ++j) {
                i64 cost = s1[i] == s2[j] ? 0 : 1;
                i64 v = std::min({at(i, j + 1) + 1, at(i + 1, j) + 1, at(i, j) + cost});
                if (i > 0 && j > 0 && s1[i] == s2[j - 1] && s1[i - 1] == s2[j]) v = std::min(v, at(i - 1, j - 1) + cost);
                at(i + 1, j + 1) = v;
            }
        return at(n1, n2);
    });
}

/* rapidfuzz_reference/Jaro.hpp:11-66 (counts only) */
void rfo_naive_jaro_counts(const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb, int64_t* common,
                           int64_t* transp)
{
    with_strs(a, la, ca, b, lb, cb, [&](auto P, auto T) -> int {
        *common = 0;
        *transp = 0;
        if (!P.n || !T.n) return 0;
        std::vector<char> pf(P.n + 1, 0), tf(T.n + 1, 0);
        i64 bound = std::max(P.n, T.n) / 2;
        if (bound > 0) --bound;
        i64 cc = 0;
        for (i64 i = 0; i < T.n; ++i) {
            i64 lo = i >= bound ? i - bound : 0;
            i64 hi = std::min(i + bound, P.n - 1);
            for (i64 j = lo; j <= hi; ++j)
                if (!pf[j] && P[j] == T[i]) {
                    tf[i] = pf[j] = 1;
                    ++cc;
                    break;
                }
        }
        i64 t = 0, k = 0;
        for (i64 i = 0; i < T.n; ++i) {
            if (!tf[i]) continue;
            i64 j = k;
            for (; j < P.n; ++j)
                if (pf[j]) {
                    k = j + 1;
                    break;
                }
            if (T[i] != P[j]) ++t;
        }
        *common = cc;
        *transp = t;
        return 0;
    });
}

int rfo_editops(int metric, const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb, uint64_t hint,
                rfo_editop* ops, int64_t cap, int64_t* count)
{
    if (metric != RFO_LEVENSHTEIN && metric != RFO_INDEL && metric != RFO_LCSSEQ) return -1;
    std::vector<rfo_editop> v;
    const int rc = with_strs(a, la, ca, b, lb, cb,
                             [&](auto s1, auto s2) -> int { return editops_impl(metric, s1, s2, hint, &v); });
    if (rc) return rc;
    *count = (int64_t)v.size();
    for (size_t k = 0; k < v.size() && (int64_t)k < cap; ++k) ops[k] = v[k];
    return 0;
}

int rfo_token_join(const void* s, int64_t len, int cw, int dedup, uint64_t* out, int64_t cap, int64_t* out_len)
{
    return with_strs(s, len, cw, s, len, cw, [&](auto a, auto) -> int {
        Tokens t = sorted_tokens(a, cw == 1);
        if (dedup) t.erase(std::unique(t.begin(), t.end()), t.end()); /* SplittedSentenceView::dedupe */
        const std::vector<u64> j = join_tokens(t);
        *out_len = (int64_t)j.size();
        for (size_t k = 0; k < j.size() && (int64_t)k < cap; ++k) out[k] = j[k];
        return 0;
    });
}

int rfo_score(int metric, int op, int form, const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb,
              const rfo_params* p, uint64_t ci, double cf, int64_t* oi, double* of)
{
    return with_strs(a, la, ca, b, lb, cb, [&](auto s1, auto s2) -> int {
        PM pm;
        pm.build(s1);
        return score_with_pm(metric, op, form, pm, s1, s2, p, ci, cf, oi, of);
    });
}

int rfo_cdist(int metric, int op, const rfo_strings* q, const rfo_strings* c, const rfo_params* p, uint64_t ci,
              double cf, int out_dtype, void* out, int nthreads)
{
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    const bool is_int = result_is_int(metric, op);
    const i64 nq = q->count, nc = c->count;
    /* work items are (query, block of choices); each item builds the query's pattern
     * once and scores the block with it (the Cached* loop of the reference) */
    const i64 CB = 2048;
    const i64 nblk = (nc + CB - 1) / CB;
    const i64 items = nq * nblk;
    std::vector<int> errs(nthreads, 0);
    std::atomic<i64> next(0);
    auto work = [&](int tid) {
        for (;;) {
            const i64 it = next.fetch_add(1);
            if (it >= items) break;
            const i64 qi = it / nblk, b0 = (it % nblk) * CB, b1 = std::min(nc, b0 + CB);
            const char* qd = (const char*)q->data + q->offsets[qi] * q->char_width;
            i64 ql = q->offsets[qi + 1] - q->offsets[qi];
            int rc = with_strs(qd, ql, q->char_width, c->data, 0, c->char_width, [&](auto s1, auto s2base) -> int {
                PM pm;
                pm.build(s1);
                for (i64 k = b0; k < b1; ++k) {
                    decltype(s2base) s2{s2base.p + c->offsets[k], c->offsets[k + 1] - c->offsets[k]};
                    i64 vi = 0;
                    double vf = 0;
                    if (score_with_pm(metric, op, RFO_FORM_CACHED, pm, s1, s2, p, ci, cf, &vi, &vf)) return -1;
                    store<int>(out, out_dtype, qi * nc + k, vi, vf, is_int);
                }
                return 0;
            });
            if (rc) errs[tid] = rc;
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
    work(0);
    for (auto& t : th) t.join();
    for (int e : errs)
        if (e) return e;
    return 0;
}

} /* extern "C" */
