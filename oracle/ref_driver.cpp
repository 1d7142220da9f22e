/*
 * ref_driver.cpp -- C entry points over the UNMODIFIED rapidfuzz-cpp headers.
 *
 * Compiled by oracle/Makefile against the reference's own sources (include path of the
 * reference checkout) into oracle/_ref/librfref.so.  It exists to pin the oracle
 * (oracle/rfo.cpp) and to generate the golden fixtures under tests/golden/; it is test
 * infrastructure, never part of the product.  The signature of rfref_score is the one of
 * rfo_score, so the same harness drives both.
 */
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <type_traits>
#include <vector>

#include <rapidfuzz/distance.hpp>
#include <rapidfuzz/fuzz.hpp>

#include "rfo.h"

namespace {

template <typename C>
std::vector<C> vec_of(const void* p, int64_t n)
{
    const C* c = static_cast<const C*>(p);
    return std::vector<C>(c, c + n);
}

template <int MaxLen, typename V1, typename V2>
int multi_call(int metric, int op, const V1& s1, const V2& s2, const rfo_params* p, uint64_t ci, double cf,
               int64_t* oi, double* of)
{
    using namespace rapidfuzz::experimental;
    auto run_int = [&](auto& scorer) {
        scorer.insert(s1);
        std::vector<size_t> r(scorer.result_count());
        if (op == RFO_DISTANCE) scorer.distance(r.data(), r.size(), s2, ci);
        else scorer.similarity(r.data(), r.size(), s2, ci);
        *oi = (int64_t)r[0];
    };
    auto run_norm = [&](auto& scorer) {
        scorer.insert(s1);
        std::vector<double> r(scorer.result_count());
        if (op == RFO_NORM_DISTANCE) scorer.normalized_distance(r.data(), r.size(), s2, cf);
        else scorer.normalized_similarity(r.data(), r.size(), s2, cf);
        *of = r[0];
    };
    auto run_f = [&](auto& scorer) {
        scorer.insert(s1);
        std::vector<double> r(scorer.result_count());
        if (op == RFO_DISTANCE) scorer.distance(r.data(), r.size(), s2, cf);
        else if (op == RFO_SIMILARITY) scorer.similarity(r.data(), r.size(), s2, cf);
        else if (op == RFO_NORM_DISTANCE) scorer.normalized_distance(r.data(), r.size(), s2, cf);
        else scorer.normalized_similarity(r.data(), r.size(), s2, cf);
        *of = r[0];
    };
    bool integral = op == RFO_DISTANCE || op == RFO_SIMILARITY;
    switch (metric) {
    case RFO_LEVENSHTEIN: {
        MultiLevenshtein<MaxLen> s(1, {(size_t)p->insert_cost, (size_t)p->delete_cost, (size_t)p->replace_cost});
        integral ? run_int(s) : run_norm(s);
        return 0;
    }
    case RFO_INDEL: {
        MultiIndel<MaxLen> s(1);
        integral ? run_int(s) : run_norm(s);
        return 0;
    }
    case RFO_LCSSEQ: {
        MultiLCSseq<MaxLen> s(1);
        integral ? run_int(s) : run_norm(s);
        return 0;
    }
    case RFO_OSA: {
        MultiOSA<MaxLen> s(1);
        integral ? run_int(s) : run_norm(s);
        return 0;
    }
    case RFO_JARO: {
        MultiJaro<MaxLen> s(1);
        run_f(s);
        return 0;
    }
    case RFO_JARO_WINKLER: {
        MultiJaroWinkler<MaxLen> s(1, p->prefix_weight);
        run_f(s);
        return 0;
    }
    case RFO_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        rapidfuzz::fuzz::experimental::MultiRatio<MaxLen> s(1);
        s.insert(s1);
        std::vector<double> r(s.result_count());
        s.similarity(r.data(), r.size(), s2, cf);
        *of = r[0];
        return 0;
    }
    }
    return -1;
}

template <typename C1, typename C2>
int score(int metric, int op, int form, const void* a, int64_t la, const void* b, int64_t lb, const rfo_params* p,
          uint64_t ci, double cf, int64_t* oi, double* of)
{
    using namespace rapidfuzz;
    std::vector<C1> s1 = vec_of<C1>(a, la);
    std::vector<C2> s2 = vec_of<C2>(b, lb);
    LevenshteinWeightTable w{(size_t)p->insert_cost, (size_t)p->delete_cost, (size_t)p->replace_cost};
    const size_t H = ci; /* score_hint follows the cutoff, like the free functions' defaults */

    if (form == RFO_FORM_MULTI) {
        if (la <= 8) return multi_call<8>(metric, op, s1, s2, p, ci, cf, oi, of);
        if (la <= 16) return multi_call<16>(metric, op, s1, s2, p, ci, cf, oi, of);
        if (la <= 32) return multi_call<32>(metric, op, s1, s2, p, ci, cf, oi, of);
        if (la <= 64) return multi_call<64>(metric, op, s1, s2, p, ci, cf, oi, of);
        return -1;
    }

    if (form == RFO_FORM_FREE) {
        switch (metric) {
        case RFO_LEVENSHTEIN:
            switch (op) {
            case RFO_DISTANCE: *oi = (int64_t)levenshtein_distance(s1, s2, w, ci, H); return 0;
            case RFO_SIMILARITY: *oi = (int64_t)levenshtein_similarity(s1, s2, w, ci, H); return 0;
            case RFO_NORM_DISTANCE: *of = levenshtein_normalized_distance(s1, s2, w, cf, cf); return 0;
            default: *of = levenshtein_normalized_similarity(s1, s2, w, cf, cf); return 0;
            }
        case RFO_INDEL:
            switch (op) {
            case RFO_DISTANCE: *oi = (int64_t)indel_distance(s1, s2, ci); return 0;
            case RFO_SIMILARITY: *oi = (int64_t)indel_similarity(s1, s2, ci); return 0;
            case RFO_NORM_DISTANCE: *of = indel_normalized_distance(s1, s2, cf); return 0;
            default: *of = indel_normalized_similarity(s1, s2, cf); return 0;
            }
        case RFO_LCSSEQ:
            switch (op) {
            case RFO_DISTANCE: *oi = (int64_t)lcs_seq_distance(s1, s2, ci); return 0;
            case RFO_SIMILARITY: *oi = (int64_t)lcs_seq_similarity(s1, s2, ci); return 0;
            case RFO_NORM_DISTANCE: *of = lcs_seq_normalized_distance(s1, s2, cf); return 0;
            default: *of = lcs_seq_normalized_similarity(s1, s2, cf); return 0;
            }
        case RFO_OSA:
            switch (op) {
            case RFO_DISTANCE: *oi = (int64_t)osa_distance(s1, s2, ci); return 0;
            case RFO_SIMILARITY: *oi = (int64_t)osa_similarity(s1, s2, ci); return 0;
            case RFO_NORM_DISTANCE: *of = osa_normalized_distance(s1, s2, cf); return 0;
            default: *of = osa_normalized_similarity(s1, s2, cf); return 0;
            }
        case RFO_JARO:
            switch (op) {
            case RFO_DISTANCE: *of = jaro_distance(s1, s2, cf); return 0;
            case RFO_SIMILARITY: *of = jaro_similarity(s1, s2, cf); return 0;
            case RFO_NORM_DISTANCE: *of = jaro_normalized_distance(s1, s2, cf); return 0;
            default: *of = jaro_normalized_similarity(s1, s2, cf); return 0;
            }
        case RFO_JARO_WINKLER:
            switch (op) {
            case RFO_DISTANCE: *of = jaro_winkler_distance(s1, s2, p->prefix_weight, cf); return 0;
            case RFO_SIMILARITY: *of = jaro_winkler_similarity(s1, s2, p->prefix_weight, cf); return 0;
            case RFO_NORM_DISTANCE: *of = jaro_winkler_normalized_distance(s1, s2, p->prefix_weight, cf); return 0;
            default: *of = jaro_winkler_normalized_similarity(s1, s2, p->prefix_weight, cf); return 0;
            }
        case RFO_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::ratio(s1, s2, cf);
            return 0;
        case RFO_PARTIAL_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::partial_ratio(s1, s2, cf);
            return 0;
        case RFO_TOKEN_SORT_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::token_sort_ratio(s1, s2, cf);
            return 0;
        case RFO_PARTIAL_TOKEN_SORT_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::partial_token_sort_ratio(s1, s2, cf);
            return 0;
        case RFO_QRATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::QRatio(s1, s2, cf);
            return 0;
        case RFO_TOKEN_SET_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::token_set_ratio(s1, s2, cf);
            return 0;
        case RFO_PARTIAL_TOKEN_SET_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::partial_token_set_ratio(s1, s2, cf);
            return 0;
        case RFO_TOKEN_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::token_ratio(s1, s2, cf);
            return 0;
        case RFO_PARTIAL_TOKEN_RATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::partial_token_ratio(s1, s2, cf);
            return 0;
        case RFO_WRATIO:
            if (op != RFO_SIMILARITY) return -1;
            *of = fuzz::WRatio(s1, s2, cf);
            return 0;
        }
        return -1;
    }

    /* cached */
    auto run_dist = [&](auto& sc) {
        switch (op) {
        case RFO_DISTANCE: *oi = (int64_t)sc.distance(s2, ci); break;
        case RFO_SIMILARITY: *oi = (int64_t)sc.similarity(s2, ci); break;
        case RFO_NORM_DISTANCE: *of = sc.normalized_distance(s2, cf); break;
        default: *of = sc.normalized_similarity(s2, cf);
        }
        return 0;
    };
    auto run_f = [&](auto& sc) {
        switch (op) {
        case RFO_DISTANCE: *of = sc.distance(s2, cf); break;
        case RFO_SIMILARITY: *of = sc.similarity(s2, cf); break;
        case RFO_NORM_DISTANCE: *of = sc.normalized_distance(s2, cf); break;
        default: *of = sc.normalized_similarity(s2, cf);
        }
        return 0;
    };
    switch (metric) {
    case RFO_LEVENSHTEIN: {
        CachedLevenshtein<C1> sc(s1, w);
        return run_dist(sc);
    }
    case RFO_INDEL: {
        CachedIndel<C1> sc(s1);
        return run_dist(sc);
    }
    case RFO_LCSSEQ: {
        CachedLCSseq<C1> sc(s1);
        return run_dist(sc);
    }
    case RFO_OSA: {
        CachedOSA<C1> sc(s1);
        return run_dist(sc);
    }
    case RFO_JARO: {
        CachedJaro<C1> sc(s1);
        return run_f(sc);
    }
    case RFO_JARO_WINKLER: {
        CachedJaroWinkler<C1> sc(s1, p->prefix_weight);
        return run_f(sc);
    }
    case RFO_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_PARTIAL_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedPartialRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_TOKEN_SORT_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedTokenSortRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_PARTIAL_TOKEN_SORT_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedPartialTokenSortRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_QRATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedQRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_TOKEN_SET_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedTokenSetRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_PARTIAL_TOKEN_SET_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedPartialTokenSetRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_TOKEN_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedTokenRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_PARTIAL_TOKEN_RATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedPartialTokenRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    case RFO_WRATIO: {
        if (op != RFO_SIMILARITY) return -1;
        fuzz::CachedWRatio<C1> sc(s1);
        *of = sc.similarity(s2, cf);
        return 0;
    }
    }
    return -1;
}

template <typename C1>
int score_c2(int metric, int op, int form, const void* a, int64_t la, const void* b, int64_t lb, int cb,
             const rfo_params* p, uint64_t ci, double cf, int64_t* oi, double* of)
{
    switch (cb) {
    case 1: return score<C1, uint8_t>(metric, op, form, a, la, b, lb, p, ci, cf, oi, of);
    case 2: return score<C1, uint16_t>(metric, op, form, a, la, b, lb, p, ci, cf, oi, of);
    case 4: return score<C1, uint32_t>(metric, op, form, a, la, b, lb, p, ci, cf, oi, of);
    default: return score<C1, uint64_t>(metric, op, form, a, la, b, lb, p, ci, cf, oi, of);
    }
}

} // namespace

extern "C" int rfref_score(int metric, int op, int form, const void* a, int64_t la, int ca, const void* b,
                           int64_t lb, int cb, const rfo_params* p, uint64_t ci, double cf, int64_t* oi,
                           double* of)
{
    try {
        switch (ca) {
        case 1: return score_c2<uint8_t>(metric, op, form, a, la, b, lb, cb, p, ci, cf, oi, of);
        case 2: return score_c2<uint16_t>(metric, op, form, a, la, b, lb, cb, p, ci, cf, oi, of);
        case 4: return score_c2<uint32_t>(metric, op, form, a, la, b, lb, cb, p, ci, cf, oi, of);
        default: return score_c2<uint64_t>(metric, op, form, a, la, b, lb, cb, p, ci, cf, oi, of);
        }
    }
    catch (const std::invalid_argument&) {
        return -1;
    }
}

/* levenshtein_editops / indel_editops / lcs_seq_editops (Levenshtein.hpp:282-295,
 * Indel.hpp:65-75, LCSseq.hpp:65-75) of the unmodified headers */
template <typename C1, typename C2>
int editops_pair(int metric, const void* a, int64_t la, const void* b, int64_t lb, uint64_t hint, rfo_editop* ops,
                 int64_t cap, int64_t* count)
{
    std::vector<C1> s1((const C1*)a, (const C1*)a + la);
    std::vector<C2> s2((const C2*)b, (const C2*)b + lb);
    rapidfuzz::Editops e;
    if (metric == RFO_LEVENSHTEIN) e = rapidfuzz::levenshtein_editops(s1, s2, (size_t)hint);
    else if (metric == RFO_INDEL) e = rapidfuzz::indel_editops(s1, s2);
    else e = rapidfuzz::lcs_seq_editops(s1, s2);
    *count = (int64_t)e.size();
    for (size_t k = 0; k < e.size() && (int64_t)k < cap; ++k)
        ops[k] = rfo_editop{(int32_t)e[k].type, 0, (int64_t)e[k].src_pos, (int64_t)e[k].dest_pos};
    return (e.get_src_len() == (size_t)la && e.get_dest_len() == (size_t)lb) ? 0 : -3;
}

template <typename C1>
int editops_c2(int metric, const void* a, int64_t la, const void* b, int64_t lb, int cb, uint64_t hint,
               rfo_editop* ops, int64_t cap, int64_t* count)
{
    switch (cb) {
    case 1: return editops_pair<C1, uint8_t>(metric, a, la, b, lb, hint, ops, cap, count);
    case 2: return editops_pair<C1, uint16_t>(metric, a, la, b, lb, hint, ops, cap, count);
    case 4: return editops_pair<C1, uint32_t>(metric, a, la, b, lb, hint, ops, cap, count);
    default: return editops_pair<C1, uint64_t>(metric, a, la, b, lb, hint, ops, cap, count);
    }
}

extern "C" int rfref_editops(int metric, const void* a, int64_t la, int ca, const void* b, int64_t lb, int cb,
                             uint64_t hint, rfo_editop* ops, int64_t cap, int64_t* count)
{
    switch (ca) {
    case 1: return editops_c2<uint8_t>(metric, a, la, b, lb, cb, hint, ops, cap, count);
    case 2: return editops_c2<uint16_t>(metric, a, la, b, lb, cb, hint, ops, cap, count);
    case 4: return editops_c2<uint32_t>(metric, a, la, b, lb, cb, hint, ops, cap, count);
    default: return editops_c2<uint64_t>(metric, a, la, b, lb, cb, hint, ops, cap, count);
    }
}

/* Opcodes(const Editops&), Editops(const Opcodes&) (details/types.hpp:500-569) and
 * editops_apply_vec / opcodes_apply_vec (distance.hpp:19-103, 134-165) of the unmodified
 * headers on one pair's operations: opc gets 5 int64 per opcode (type, src_begin, src_end,
 * dest_begin, dest_end), back the editops of those opcodes, ea / oa (room for la + lb
 * units) the two applies of s1 (a, la units) and s2 (b, lb units), one-byte strings.
 * Counts are always written; entries up to the capacities. */
extern "C" int rfref_opcodes(const rfo_editop* ops, int64_t n, const void* a, int64_t la, const void* b, int64_t lb,
                             int64_t* opc, int64_t cap, int64_t* count, rfo_editop* back, int64_t bcap,
                             int64_t* bcount, uint8_t* ea, int64_t* ea_len, uint8_t* oa, int64_t* oa_len)
{
    rapidfuzz::Editops e((size_t)n);
    for (int64_t k = 0; k < n; ++k)
        e[(size_t)k] = rapidfuzz::EditOp((rapidfuzz::EditType)ops[k].type, (size_t)ops[k].src_pos,
                                         (size_t)ops[k].dest_pos);
    e.set_src_len((size_t)la);
    e.set_dest_len((size_t)lb);
    const rapidfuzz::Opcodes o(e);
    *count = (int64_t)o.size();
    for (size_t k = 0; k < o.size() && (int64_t)k < cap; ++k) {
        int64_t* r = opc + 5 * k;
        r[0] = (int64_t)o[k].type;
        r[1] = (int64_t)o[k].src_begin;
        r[2] = (int64_t)o[k].src_end;
        r[3] = (int64_t)o[k].dest_begin;
        r[4] = (int64_t)o[k].dest_end;
    }
    const rapidfuzz::Editops bk(o);
    *bcount = (int64_t)bk.size();
    for (size_t k = 0; k < bk.size() && (int64_t)k < bcap; ++k)
        back[k] = rfo_editop{(int32_t)bk[k].type, 0, (int64_t)bk[k].src_pos, (int64_t)bk[k].dest_pos};
    const std::vector<uint8_t> s1((const uint8_t*)a, (const uint8_t*)a + la), s2((const uint8_t*)b, (const uint8_t*)b + lb);
    const std::vector<uint8_t> x = rapidfuzz::editops_apply_vec<uint8_t>(e, s1, s2);
    const std::vector<uint8_t> y = rapidfuzz::opcodes_apply_vec<uint8_t>(o, s1, s2);
    *ea_len = (int64_t)x.size();
    *oa_len = (int64_t)y.size();
    std::copy(x.begin(), x.end(), ea);
    std::copy(y.begin(), y.end(), oa);
    return 0;
}

/* the list operations of Editops / Opcodes (details/types.hpp:109-161, 240-320, 420-475)
 * of the unmodified headers on one operation list: which 0 Editops::slice, 1
 * remove_slice, 2 reverse, 3 inverse, 4 remove_subsequence(slice(start, stop, step)); 10
 * Opcodes(ops).slice, 12 reverse, 13 inverse.  out gets 3
 * int64 per edit operation or 5 per opcode (up to cap records), lens the result's
 * src_len / dest_len.  Returns 0, or -1 where the reference throws invalid_argument. */
extern "C" int rfref_list_op(int which, const rfo_editop* ops, int64_t n, int64_t src_len, int64_t dest_len, int start,
                             int stop, int step, int64_t* out, int64_t cap, int64_t* count, int64_t* lens)
{
    rapidfuzz::Editops e((size_t)n);
    for (int64_t k = 0; k < n; ++k)
        e[(size_t)k] = rapidfuzz::EditOp((rapidfuzz::EditType)ops[k].type, (size_t)ops[k].src_pos,
                                         (size_t)ops[k].dest_pos);
    e.set_src_len((size_t)src_len);
    e.set_dest_len((size_t)dest_len);
    try {
        if (which < 10) {
            rapidfuzz::Editops r;
            if (which == 0) r = e.slice(start, stop, step);
            else if (which == 1) {
                r = e;
                r.remove_slice(start, stop, step);
            }
            else if (which == 2) r = e.reverse();
            else if (which == 3) r = e.inverse();
            else r = e.remove_subsequence(e.slice(start, stop, step));
            *count = (int64_t)r.size();
            for (size_t k = 0; k < r.size() && (int64_t)k < cap; ++k) {
                out[3 * k] = (int64_t)r[k].type;
                out[3 * k + 1] = (int64_t)r[k].src_pos;
                out[3 * k + 2] = (int64_t)r[k].dest_pos;
            }
            lens[0] = (int64_t)r.get_src_len();
            lens[1] = (int64_t)r.get_dest_len();
            return 0;
        }
        const rapidfuzz::Opcodes o(e);
        rapidfuzz::Opcodes r;
        if (which == 10) r = o.slice(start, stop, step);
        else if (which == 12) r = o.reverse();
        else r = o.inverse();
        *count = (int64_t)r.size();
        for (size_t k = 0; k < r.size() && (int64_t)k < cap; ++k) {
            out[5 * k] = (int64_t)r[k].type;
            out[5 * k + 1] = (int64_t)r[k].src_begin;
            out[5 * k + 2] = (int64_t)r[k].src_end;
            out[5 * k + 3] = (int64_t)r[k].dest_begin;
            out[5 * k + 4] = (int64_t)r[k].dest_end;
        }
        lens[0] = (int64_t)r.get_src_len();
        lens[1] = (int64_t)r.get_dest_len();
        return 0;
    }
    catch (const std::invalid_argument&) {
        return -1;
    }
}

/* Multi* with several inserted strings (padding semantics, result order) */
extern "C" int rfref_multi(int metric, int op, int max_len, const rfo_strings* inserted, const void* b, int64_t lb,
                           int cb, const rfo_params* p, uint64_t ci, double cf, int64_t* oi, double* of,
                           int64_t* result_count)
{
    (void)cb;
    if (inserted->char_width != 1 || cb != 1) return -2;
    std::vector<std::vector<uint8_t>> strs;
    for (int64_t i = 0; i < inserted->count; ++i) {
        const uint8_t* d = (const uint8_t*)inserted->data + inserted->offsets[i];
        strs.emplace_back(d, d + (inserted->offsets[i + 1] - inserted->offsets[i]));
    }
    std::vector<uint8_t> s2((const uint8_t*)b, (const uint8_t*)b + lb);
    using namespace rapidfuzz::experimental;
    auto go = [&](auto& sc, auto fl) {
        for (auto& s : strs) sc.insert(s);
        *result_count = (int64_t)sc.result_count();
        if (!oi && !of) return 0;
        if constexpr (!decltype(fl)::value) {
            if (op == RFO_DISTANCE || op == RFO_SIMILARITY) {
                std::vector<size_t> r(sc.result_count());
                if (op == RFO_DISTANCE) sc.distance(r.data(), r.size(), s2, ci);
                else sc.similarity(r.data(), r.size(), s2, ci);
                for (size_t i = 0; i < strs.size(); ++i) oi[i] = (int64_t)r[i];
            }
            else {
                std::vector<double> r(sc.result_count());
                if (op == RFO_NORM_DISTANCE) sc.normalized_distance(r.data(), r.size(), s2, cf);
                else sc.normalized_similarity(r.data(), r.size(), s2, cf);
                for (size_t i = 0; i < strs.size(); ++i) of[i] = r[i];
            }
        }
        else {
            std::vector<double> r(sc.result_count());
            if (op == RFO_NORM_DISTANCE) sc.normalized_distance(r.data(), r.size(), s2, cf);
            else if (op == RFO_NORM_SIMILARITY) sc.normalized_similarity(r.data(), r.size(), s2, cf);
            else if (op == RFO_DISTANCE) sc.distance(r.data(), r.size(), s2, cf);
            else sc.similarity(r.data(), r.size(), s2, cf);
            for (size_t i = 0; i < strs.size(); ++i) of[i] = r[i];
        }
        return 0;
    };
    /* the fuzz Multi scorers: similarity only */
    auto fuzz_go = [&](auto& sc) {
        for (auto& x : strs) sc.insert(x);
        *result_count = (int64_t)sc.result_count();
        if (!of) return 0;
        std::vector<double> r(sc.result_count());
        sc.similarity(r.data(), r.size(), s2, cf);
        for (size_t i = 0; i < strs.size(); ++i) of[i] = r[i];
        return 0;
    };
    try {
#define RF_MULTI_CASE(ML)                                                                                      \
    case ML:                                                                                                   \
        switch (metric) {                                                                                      \
        case RFO_LEVENSHTEIN: {                                                                                \
            MultiLevenshtein<ML> s(strs.size(), {(size_t)p->insert_cost, (size_t)p->delete_cost,               \
                                                 (size_t)p->replace_cost});                                    \
            return go(s, std::false_type{});                                                                               \
        }                                                                                                      \
        case RFO_INDEL: {                                                                                      \
            MultiIndel<ML> s(strs.size());                                                                     \
            return go(s, std::false_type{});                                                                               \
        }                                                                                                      \
        case RFO_LCSSEQ: {                                                                                     \
            MultiLCSseq<ML> s(strs.size());                                                                    \
            return go(s, std::false_type{});                                                                               \
        }                                                                                                      \
        case RFO_OSA: {                                                                                        \
            MultiOSA<ML> s(strs.size());                                                                       \
            return go(s, std::false_type{});                                                                               \
        }                                                                                                      \
        case RFO_JARO: {                                                                                       \
            MultiJaro<ML> s(strs.size());                                                                      \
            return go(s, std::true_type{});                                                                                \
        }                                                                                                      \
        case RFO_JARO_WINKLER: {                                                                               \
            MultiJaroWinkler<ML> s(strs.size(), p->prefix_weight);                                             \
            return go(s, std::true_type{});                                                                                \
        }                                                                                                      \
        case RFO_RATIO: {                                                                                      \
            rapidfuzz::fuzz::experimental::MultiRatio<ML> s(strs.size());                                      \
            return fuzz_go(s);                                                                                 \
        }                                                                                                      \
        case RFO_TOKEN_SORT_RATIO: {                                                                           \
            rapidfuzz::fuzz::experimental::MultiTokenSortRatio<ML> s(strs.size());                             \
            return fuzz_go(s);                                                                                 \
        }                                                                                                      \
        case RFO_QRATIO: {                                                                                     \
            rapidfuzz::fuzz::experimental::MultiQRatio<ML> s(strs.size());                                     \
            return fuzz_go(s);                                                                                 \
        }                                                                                                      \
        }                                                                                                      \
        return -1;
        switch (max_len) {
            RF_MULTI_CASE(8)
            RF_MULTI_CASE(16)
            RF_MULTI_CASE(32)
            RF_MULTI_CASE(64)
        }
#undef RF_MULTI_CASE
    }
    catch (const std::invalid_argument&) {
        return -1;
    }
    return -1;
}
