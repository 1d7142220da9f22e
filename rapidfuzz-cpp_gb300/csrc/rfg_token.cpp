/* Host front end of the token scorers: sorted_split(s).join() of the strings before the
 * ratio / partial_ratio engine scores them (fuzz_impl.hpp:294-360).  Host code only. */
#include "rfg_token.h"

#include <string.h>

#include <algorithm>
#include <thread>
#include <utility>

namespace rfg {
namespace {

/* is_space (common_impl.hpp:85-152) */
template <typename T>
bool is_ws(T c)
{
    switch ((uint64_t)c) {
    case 0x09: case 0x0A: case 0x0B: case 0x0C: case 0x0D: case 0x1C: case 0x1D: case 0x1E: case 0x1F:
    case 0x20: return true;
    }
    if (sizeof(T) == 1) return false;
    switch ((uint64_t)c) {
    case 0x85: case 0xA0: case 0x1680: case 0x2000: case 0x2001: case 0x2002: case 0x2003: case 0x2004:
    case 0x2005: case 0x2006: case 0x2007: case 0x2008: case 0x2009: case 0x200A: case 0x2028: case 0x2029:
    case 0x202F: case 0x205F: case 0x3000: return true;
    }
    return false;
}

using Tokens = std::vector<std::pair<int64_t, int64_t>>; /* [begin, end) */

/* joins s[0, n) into out (room for n units: the join is never longer than the string) */
template <typename T>
int64_t join_into(const T* s, int64_t n, T* out, Tokens& tok)
{
    tok.clear();
    for (int64_t i = 0; i < n;) {
        while (i < n && is_ws(s[i])) ++i;
        const int64_t a = i;
        while (i < n && !is_ws(s[i])) ++i;
        if (i > a) tok.emplace_back(a, i);
    }
    /* equal tokens are equal sequences, so an unstable sort gives the same join */
    std::sort(tok.begin(), tok.end(), [s](const std::pair<int64_t, int64_t>& x, const std::pair<int64_t, int64_t>& y) {
        return std::lexicographical_compare(s + x.first, s + x.second, s + y.first, s + y.second);
    });
    int64_t w = 0;
    for (size_t k = 0; k < tok.size(); ++k) {
        if (k) out[w++] = (T)0x20;
        for (int64_t i = tok[k].first; i < tok[k].second; ++i) out[w++] = s[i];
    }
    return w;
}

template <typename F>
void parallel_ranges(int64_t n, int64_t grain, F f)
{
    const int64_t hw = std::max<int64_t>(1, (int64_t)std::thread::hardware_concurrency());
    const int64_t nt = std::min<int64_t>(std::min<int64_t>(hw, 64), std::max<int64_t>(1, n / grain));
    if (nt <= 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < nt; ++t) th.emplace_back(f, n * t / nt, n * (t + 1) / nt);
    for (auto& x : th) x.join();
}

template <typename T>
void join_set(const T* data, const int64_t* off, int64_t n, std::vector<unsigned char>* od, std::vector<int64_t>* oo)
{
    const int64_t base = n ? off[0] : 0, total = n ? off[n] - base : 0;
    std::vector<T> tmp((size_t)total);
    std::vector<int64_t> jl((size_t)n);
    /* pass 1: each join at its string's own position (it fits there) */
    parallel_ranges(n, 4096, [&](int64_t a, int64_t b) {
        Tokens tok;
        for (int64_t i = a; i < b; ++i)
            jl[i] = join_into(data + off[i], off[i + 1] - off[i], tmp.data() + (off[i] - base), tok);
    });
    oo->assign((size_t)n + 1, 0);
    for (int64_t i = 0; i < n; ++i) (*oo)[i + 1] = (*oo)[i] + jl[i];
    od->assign((size_t)(*oo)[n] * sizeof(T) + 16, 0);
    T* dst = (T*)od->data();
    /* pass 2: pack */
    parallel_ranges(n, 16384, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i)
            if (jl[i]) memcpy(dst + (*oo)[i], tmp.data() + (off[i] - base), (size_t)jl[i] * sizeof(T));
    });
}

/* [s][S][J] parts of one string into out (room for 3 n units); lens gets the three lengths */
template <typename T>
int64_t parts_into(const T* s, int64_t n, bool orig, bool sorted, bool dedup, T* out, Tokens& tok, int32_t* lens)
{
    int64_t w = 0;
    lens[0] = lens[1] = lens[2] = 0;
    if (orig) {
        for (int64_t i = 0; i < n; ++i) out[w++] = s[i];
        lens[0] = (int32_t)n;
    }
    if (!sorted && !dedup) return w;
    const int64_t ls = join_into(s, n, out + w, tok); /* tok: the sorted tokens */
    if (sorted) {
        lens[1] = (int32_t)ls;
        w += ls;
    }
    if (dedup) {
        int64_t wj = 0;
        for (size_t k = 0; k < tok.size(); ++k) {
            if (k && std::equal(s + tok[k].first, s + tok[k].second, s + tok[k - 1].first, s + tok[k - 1].second))
                continue;
            if (wj) out[w + wj++] = (T)0x20;
            for (int64_t i = tok[k].first; i < tok[k].second; ++i) out[w + wj++] = s[i];
        }
        lens[2] = (int32_t)wj;
        w += wj;
    }
    return w;
}

template <typename T>
void parts_set(const T* data, const int64_t* off, int64_t n, bool orig, bool sorted, bool dedup,
               std::vector<unsigned char>* od, std::vector<int64_t>* oo, std::vector<int32_t>* parts)
{
    const int64_t base = n ? off[0] : 0, total = n ? off[n] - base : 0;
    std::vector<T> tmp((size_t)(3 * total));
    std::vector<int64_t> jl((size_t)n);
    parts->assign((size_t)(3 * n), 0);
    parallel_ranges(n, 4096, [&](int64_t a, int64_t b) {
        Tokens tok;
        for (int64_t i = a; i < b; ++i)
            jl[i] = parts_into(data + off[i], off[i + 1] - off[i], orig, sorted, dedup, tmp.data() + 3 * (off[i] - base),
                               tok, parts->data() + 3 * i);
    });
    oo->assign((size_t)n + 1, 0);
    for (int64_t i = 0; i < n; ++i) (*oo)[i + 1] = (*oo)[i] + jl[i];
    od->assign((size_t)(*oo)[n] * sizeof(T) + 16, 0);
    T* dst = (T*)od->data();
    parallel_ranges(n, 16384, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i)
            if (jl[i]) memcpy(dst + (*oo)[i], tmp.data() + 3 * (off[i] - base), (size_t)jl[i] * sizeof(T));
    });
}

template <typename T>
int64_t join_one(const void* s, int64_t len, std::vector<unsigned char>* out)
{
    out->assign((size_t)len * sizeof(T) + 16, 0);
    Tokens tok;
    return join_into((const T*)s, len, (T*)out->data(), tok);
}

} // namespace

void token_parts_set(const void* data, const int64_t* off, int64_t n, int width, bool orig, bool sorted, bool dedup,
                     std::vector<unsigned char>* out_data, std::vector<int64_t>* out_off, std::vector<int32_t>* parts)
{
    switch (width) {
    case 1: parts_set((const uint8_t*)data, off, n, orig, sorted, dedup, out_data, out_off, parts); break;
    case 2: parts_set((const uint16_t*)data, off, n, orig, sorted, dedup, out_data, out_off, parts); break;
    case 4: parts_set((const uint32_t*)data, off, n, orig, sorted, dedup, out_data, out_off, parts); break;
    default: parts_set((const uint64_t*)data, off, n, orig, sorted, dedup, out_data, out_off, parts); break;
    }
}

int64_t token_sort_join(const void* s, int64_t len, int width, std::vector<unsigned char>* out)
{
    switch (width) {
    case 1: return join_one<uint8_t>(s, len, out);
    case 2: return join_one<uint16_t>(s, len, out);
    case 4: return join_one<uint32_t>(s, len, out);
    default: return join_one<uint64_t>(s, len, out);
    }
}

void token_sort_join_set(const void* data, const int64_t* off, int64_t n, int width,
                         std::vector<unsigned char>* out_data, std::vector<int64_t>* out_off)
{
    switch (width) {
    case 1: join_set((const uint8_t*)data, off, n, out_data, out_off); break;
    case 2: join_set((const uint16_t*)data, off, n, out_data, out_off); break;
    case 4: join_set((const uint32_t*)data, off, n, out_data, out_off); break;
    default: join_set((const uint64_t*)data, off, n, out_data, out_off); break;
    }
}

} // namespace rfg
