/*
 * rapidfuzz_gb300/rapidfuzz.hpp -- the rapidfuzz-cpp API over the GB300 library.
 *
 * Same names, overloads, defaults and exceptions as rapidfuzz-cpp v3.3.3 (paths relative
 * to that project), in namespace rapidfuzz_gb300; a caller switches with
 *     namespace rapidfuzz = rapidfuzz_gb300;
 * and links librapidfuzz_gb300.so.  Every call runs on the GPU through the C ABI in
 * rapidfuzz_gb300.h; results are the reference's (integers bit-exact, doubles
 * bit-identical).
 *
 *   free functions   rapidfuzz/distance/{Levenshtein,Indel,LCSseq,OSA,Jaro,JaroWinkler}.hpp
 *   Cached* scorers  same files (CachedLevenshtein Levenshtein.hpp:421-482, ...)
 *   Multi* scorers   experimental::Multi*<MaxLen> (Levenshtein.hpp:297-419, ...)
 *   fuzz::ratio      rapidfuzz/fuzz.hpp:44-126 (and CachedRatio, experimental::MultiRatio)
 *   fuzz::partial_ratio, token_sort_ratio, partial_token_sort_ratio, token_set_ratio,
 *   partial_token_set_ratio, token_ratio, partial_token_ratio, WRatio, QRatio
 *                    rapidfuzz/fuzz.hpp:128-804 (Cached*, MultiTokenSortRatio, MultiQRatio)
 * Exceptions: std::invalid_argument where the reference throws it; std::runtime_error
 * for device failures (the reference has none).
 */
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <iterator>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "rapidfuzz_gb300.h"

namespace rapidfuzz_gb300 {

/* rapidfuzz/details/types.hpp:19-23 */
struct LevenshteinWeightTable {
    size_t insert_cost;
    size_t delete_cost;
    size_t replace_cost;
};

namespace detail {

inline void throw_on(rfg_status s)
{
    if (s == RFG_OK) return;
    const char* msg = rfg_last_error();
    if (s == RFG_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    if (s == RFG_ERR_OUT_OF_RANGE) throw std::out_of_range(msg);
    throw std::runtime_error(std::string("rapidfuzz_gb300: ") + msg);
}

/* a string as unsigned code units: contiguous storage is referenced, anything else copied */
template <typename T>
struct Units {
    const void* data = nullptr;
    int64_t len = 0;
    int32_t width = 1;
    std::vector<typename std::make_unsigned<T>::type> copy;
};

template <typename T>
struct is_unit : std::integral_constant<bool, std::is_integral<T>::value && !std::is_same<T, bool>::value &&
                                                  (sizeof(T) == 1 || sizeof(T) == 2 || sizeof(T) == 4 ||
                                                   sizeof(T) == 8)> {};

/* iterator overloads only take part for iterator types (no clash with Sentence + weights) */
template <typename T, typename = void>
struct is_iter : std::false_type {};
template <typename T>
struct is_iter<T, decltype(void(std::declval<typename std::iterator_traits<T>::iterator_category>()))>
    : std::true_type {};
template <typename T>
using if_iter = typename std::enable_if<is_iter<T>::value, int>::type;
template <typename T>
using if_not_array = typename std::enable_if<!std::is_array<T>::value && !std::is_pointer<T>::value, int>::type;

template <typename InputIt>
Units<typename std::iterator_traits<InputIt>::value_type> units(InputIt first, InputIt last)
{
    using T = typename std::iterator_traits<InputIt>::value_type;
    static_assert(is_unit<T>::value, "code units must be integral types of 1, 2, 4 or 8 bytes");
    Units<T> u;
    for (; first != last; ++first) u.copy.push_back(static_cast<typename std::make_unsigned<T>::type>(*first));
    u.data = u.copy.data();
    u.len = (int64_t)u.copy.size();
    u.width = (int32_t)sizeof(T);
    return u;
}

template <typename Sentence, if_not_array<Sentence> = 0>
auto units(const Sentence& s) -> Units<typename std::decay<decltype(*std::begin(s))>::type>
{
    using T = typename std::decay<decltype(*std::begin(s))>::type;
    static_assert(is_unit<T>::value, "code units must be integral types of 1, 2, 4 or 8 bytes");
    Units<T> u;
    const auto n = std::distance(std::begin(s), std::end(s));
    if (n > 0 && std::is_pointer<decltype(&*std::begin(s))>::value &&
        &*std::begin(s) + (n - 1) == &*std::prev(std::end(s))) {
        u.data = static_cast<const void*>(&*std::begin(s));
        u.len = (int64_t)n;
    }
    else {
        for (const auto& ch : s) u.copy.push_back(static_cast<typename std::make_unsigned<T>::type>(ch));
        u.data = u.copy.data();
        u.len = (int64_t)u.copy.size();
    }
    u.width = (int32_t)sizeof(T);
    return u;
}

/* NUL-terminated strings and string literals: the characters before the first NUL */
template <typename CharT>
Units<CharT> units(const CharT* s)
{
    Units<CharT> u;
    int64_t n = 0;
    while (s[n] != 0) ++n;
    u.data = s;
    u.len = n;
    u.width = (int32_t)sizeof(CharT);
    return u;
}


inline rfg_params lev_params(LevenshteinWeightTable w)
{
    return rfg_params{(int64_t)w.insert_cost, (int64_t)w.delete_cost, (int64_t)w.replace_cost, 0.1};
}

inline rfg_params jw_params(double pw) { return rfg_params{1, 1, 1, pw}; }

template <typename U1, typename U2>
size_t score_i(rfg_metric m, rfg_op op, const U1& a, const U2& b, const rfg_params& p, size_t cutoff, size_t hint)
{
    int64_t r = 0;
    throw_on(rfg_score_i64(m, op, a.data, a.len, a.width, b.data, b.len, b.width, &p, cutoff, hint, &r));
    return (size_t)r;
}

template <typename U1, typename U2>
double score_f(rfg_metric m, rfg_op op, const U1& a, const U2& b, const rfg_params& p, double cutoff, double hint)
{
    double r = 0;
    throw_on(rfg_score_f64(m, op, a.data, a.len, a.width, b.data, b.len, b.width, &p, cutoff, hint, &r));
    return r;
}

/* the integer defaults of the reference: distance cutoff SIZE_MAX, similarity 0 */
constexpr size_t SIZE_MAX_ = std::numeric_limits<size_t>::max();

} // namespace detail

/* -------------------------------------------------------------- free functions */

#define RFG_FREE_INT(NAME, METRIC, OP, DEFCUT)                                                                 \
    template <typename Sentence1, typename Sentence2>                                                          \
    size_t NAME(const Sentence1& s1, const Sentence2& s2, size_t score_cutoff = DEFCUT)                        \
    {                                                                                                          \
        return detail::score_i(METRIC, OP, detail::units(s1), detail::units(s2), rfg_params{1, 1, 1, 0.1},     \
                               score_cutoff, score_cutoff);                                                    \
    }                                                                                                          \
    template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>                              \
    size_t NAME(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2, size_t score_cutoff = DEFCUT) \
    {                                                                                                          \
        return detail::score_i(METRIC, OP, detail::units(first1, last1), detail::units(first2, last2),         \
                               rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);                          \
    }

#define RFG_FREE_DBL(NAME, METRIC, OP, DEFCUT)                                                                 \
    template <typename Sentence1, typename Sentence2>                                                          \
    double NAME(const Sentence1& s1, const Sentence2& s2, double score_cutoff = DEFCUT)                        \
    {                                                                                                          \
        return detail::score_f(METRIC, OP, detail::units(s1), detail::units(s2), rfg_params{1, 1, 1, 0.1},     \
                               score_cutoff, score_cutoff);                                                    \
    }                                                                                                          \
    template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>                              \
    double NAME(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2, double score_cutoff = DEFCUT) \
    {                                                                                                          \
        return detail::score_f(METRIC, OP, detail::units(first1, last1), detail::units(first2, last2),         \
                               rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);                          \
    }

/* Indel.hpp:12-63, LCSseq.hpp:12-63, OSA.hpp:12-111, Jaro.hpp:12-61 */
RFG_FREE_INT(indel_distance, RFG_INDEL, RFG_DISTANCE, detail::SIZE_MAX_)
RFG_FREE_INT(indel_similarity, RFG_INDEL, RFG_SIMILARITY, 0)
RFG_FREE_DBL(indel_normalized_distance, RFG_INDEL, RFG_NORMALIZED_DISTANCE, 1.0)
RFG_FREE_DBL(indel_normalized_similarity, RFG_INDEL, RFG_NORMALIZED_SIMILARITY, 0.0)
RFG_FREE_INT(lcs_seq_distance, RFG_LCSSEQ, RFG_DISTANCE, detail::SIZE_MAX_)
RFG_FREE_INT(lcs_seq_similarity, RFG_LCSSEQ, RFG_SIMILARITY, 0)
RFG_FREE_DBL(lcs_seq_normalized_distance, RFG_LCSSEQ, RFG_NORMALIZED_DISTANCE, 1.0)
RFG_FREE_DBL(lcs_seq_normalized_similarity, RFG_LCSSEQ, RFG_NORMALIZED_SIMILARITY, 0.0)
RFG_FREE_INT(osa_distance, RFG_OSA, RFG_DISTANCE, detail::SIZE_MAX_)
RFG_FREE_INT(osa_similarity, RFG_OSA, RFG_SIMILARITY, 0)
RFG_FREE_DBL(osa_normalized_distance, RFG_OSA, RFG_NORMALIZED_DISTANCE, 1.0)
RFG_FREE_DBL(osa_normalized_similarity, RFG_OSA, RFG_NORMALIZED_SIMILARITY, 0.0)
RFG_FREE_DBL(jaro_distance, RFG_JARO, RFG_DISTANCE, 1.0)
RFG_FREE_DBL(jaro_similarity, RFG_JARO, RFG_SIMILARITY, 0.0)
RFG_FREE_DBL(jaro_normalized_distance, RFG_JARO, RFG_NORMALIZED_DISTANCE, 1.0)
RFG_FREE_DBL(jaro_normalized_similarity, RFG_JARO, RFG_NORMALIZED_SIMILARITY, 0.0)

#undef RFG_FREE_INT
#undef RFG_FREE_DBL

/* Levenshtein.hpp:140-265: weights, score_cutoff, score_hint */
template <typename Sentence1, typename Sentence2>
size_t levenshtein_distance(const Sentence1& s1, const Sentence2& s2, LevenshteinWeightTable weights = {1, 1, 1},
                            size_t score_cutoff = detail::SIZE_MAX_, size_t score_hint = detail::SIZE_MAX_)
{
    return detail::score_i(RFG_LEVENSHTEIN, RFG_DISTANCE, detail::units(s1), detail::units(s2),
                           detail::lev_params(weights), score_cutoff, score_hint);
}
template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>
size_t levenshtein_distance(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2,
                            LevenshteinWeightTable weights = {1, 1, 1}, size_t score_cutoff = detail::SIZE_MAX_,
                            size_t score_hint = detail::SIZE_MAX_)
{
    return detail::score_i(RFG_LEVENSHTEIN, RFG_DISTANCE, detail::units(first1, last1), detail::units(first2, last2),
                           detail::lev_params(weights), score_cutoff, score_hint);
}
template <typename Sentence1, typename Sentence2>
size_t levenshtein_similarity(const Sentence1& s1, const Sentence2& s2, LevenshteinWeightTable weights = {1, 1, 1},
                              size_t score_cutoff = 0, size_t score_hint = 0)
{
    return detail::score_i(RFG_LEVENSHTEIN, RFG_SIMILARITY, detail::units(s1), detail::units(s2),
                           detail::lev_params(weights), score_cutoff, score_hint);
}
template <typename Sentence1, typename Sentence2>
double levenshtein_normalized_distance(const Sentence1& s1, const Sentence2& s2,
                                       LevenshteinWeightTable weights = {1, 1, 1}, double score_cutoff = 1.0,
                                       double score_hint = 1.0)
{
    return detail::score_f(RFG_LEVENSHTEIN, RFG_NORMALIZED_DISTANCE, detail::units(s1), detail::units(s2),
                           detail::lev_params(weights), score_cutoff, score_hint);
}
template <typename Sentence1, typename Sentence2>
double levenshtein_normalized_similarity(const Sentence1& s1, const Sentence2& s2,
                                         LevenshteinWeightTable weights = {1, 1, 1}, double score_cutoff = 0.0,
                                         double score_hint = 0.0)
{
    return detail::score_f(RFG_LEVENSHTEIN, RFG_NORMALIZED_SIMILARITY, detail::units(s1), detail::units(s2),
                           detail::lev_params(weights), score_cutoff, score_hint);
}

/* JaroWinkler.hpp:11-73: prefix_weight, score_cutoff */
#define RFG_JW(NAME, OP, DEFCUT)                                                                               \
    template <typename Sentence1, typename Sentence2>                                                          \
    double NAME(const Sentence1& s1, const Sentence2& s2, double prefix_weight = 0.1, double score_cutoff = DEFCUT) \
    {                                                                                                          \
        return detail::score_f(RFG_JARO_WINKLER, OP, detail::units(s1), detail::units(s2),                     \
                               detail::jw_params(prefix_weight), score_cutoff, score_cutoff);                  \
    }
RFG_JW(jaro_winkler_distance, RFG_DISTANCE, 1.0)
RFG_JW(jaro_winkler_similarity, RFG_SIMILARITY, 0.0)
RFG_JW(jaro_winkler_normalized_distance, RFG_NORMALIZED_DISTANCE, 1.0)
RFG_JW(jaro_winkler_normalized_similarity, RFG_NORMALIZED_SIMILARITY, 0.0)
#undef RFG_JW

/* ------------------------------------------------------------------ Cached* */

namespace detail {

/* CachedDistanceBase / CachedSimilarityBase / CachedNormalizedMetricBase (distance.hpp:210-388) */
class CachedScorer {
public:
    CachedScorer(const CachedScorer&) = delete;
    CachedScorer& operator=(const CachedScorer&) = delete;
    ~CachedScorer()
    {
        if (h_) rfg_cached_destroy(h_);
    }

protected:
    template <typename U>
    CachedScorer(rfg_metric m, const U& s1, const rfg_params& p) : metric_(m)
    {
        throw_on(rfg_cached_create(m, s1.data, s1.len, s1.width, &p, &h_));
    }
    template <typename U>
    size_t cached_i(rfg_op op, const U& s2, size_t cutoff, size_t hint) const
    {
        int64_t r = 0;
        throw_on(rfg_cached_score_i64(h_, op, s2.data, s2.len, s2.width, cutoff, hint, &r));
        return (size_t)r;
    }
    template <typename U>
    double cached_f(rfg_op op, const U& s2, double cutoff, double hint) const
    {
        double r = 0;
        throw_on(rfg_cached_score_f64(h_, op, s2.data, s2.len, s2.width, cutoff, hint, &r));
        return r;
    }
    rfg_metric metric_;
    rfg_cached h_ = nullptr;
};

/* integer-valued metrics: distance/similarity as size_t, normalized as double */
class CachedIntScorer : public CachedScorer {
public:
    template <typename Sentence2>
    size_t distance(const Sentence2& s2, size_t score_cutoff = SIZE_MAX_default(), size_t score_hint = SIZE_MAX_default()) const
    {
        return cached_i(RFG_DISTANCE, units(s2), score_cutoff, score_hint);
    }
    template <typename InputIt2, rapidfuzz_gb300::detail::if_iter<InputIt2> = 0>
    size_t distance(InputIt2 first2, InputIt2 last2, size_t score_cutoff = SIZE_MAX_default(),
                    size_t score_hint = SIZE_MAX_default()) const
    {
        return cached_i(RFG_DISTANCE, units(first2, last2), score_cutoff, score_hint);
    }
    template <typename Sentence2>
    size_t similarity(const Sentence2& s2, size_t score_cutoff = 0, size_t score_hint = 0) const
    {
        return cached_i(RFG_SIMILARITY, units(s2), score_cutoff, score_hint);
    }
    template <typename InputIt2, rapidfuzz_gb300::detail::if_iter<InputIt2> = 0>
    size_t similarity(InputIt2 first2, InputIt2 last2, size_t score_cutoff = 0, size_t score_hint = 0) const
    {
        return cached_i(RFG_SIMILARITY, units(first2, last2), score_cutoff, score_hint);
    }
    template <typename Sentence2>
    double normalized_distance(const Sentence2& s2, double score_cutoff = 1.0, double score_hint = 1.0) const
    {
        return cached_f(RFG_NORMALIZED_DISTANCE, units(s2), score_cutoff, score_hint);
    }
    template <typename Sentence2>
    double normalized_similarity(const Sentence2& s2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_NORMALIZED_SIMILARITY, units(s2), score_cutoff, score_hint);
    }

protected:
    /* WorstDistance of the Cached* bases: INT64_MAX (Levenshtein.hpp:422-423) */
    static constexpr size_t SIZE_MAX_default() { return (size_t)std::numeric_limits<int64_t>::max(); }
    template <typename U>
    CachedIntScorer(rfg_metric m, const U& s1, const rfg_params& p) : CachedScorer(m, s1, p)
    {}
};

/* double-valued metrics (Jaro, Jaro-Winkler) */
class CachedDblScorer : public CachedScorer {
public:
    template <typename Sentence2>
    double distance(const Sentence2& s2, double score_cutoff = 1.0, double score_hint = 1.0) const
    {
        return cached_f(RFG_DISTANCE, units(s2), score_cutoff, score_hint);
    }
    template <typename Sentence2>
    double similarity(const Sentence2& s2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_SIMILARITY, units(s2), score_cutoff, score_hint);
    }
    template <typename InputIt2, rapidfuzz_gb300::detail::if_iter<InputIt2> = 0>
    double similarity(InputIt2 first2, InputIt2 last2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_SIMILARITY, units(first2, last2), score_cutoff, score_hint);
    }
    template <typename Sentence2>
    double normalized_distance(const Sentence2& s2, double score_cutoff = 1.0, double score_hint = 1.0) const
    {
        return cached_f(RFG_NORMALIZED_DISTANCE, units(s2), score_cutoff, score_hint);
    }
    template <typename Sentence2>
    double normalized_similarity(const Sentence2& s2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_NORMALIZED_SIMILARITY, units(s2), score_cutoff, score_hint);
    }

protected:
    template <typename U>
    CachedDblScorer(rfg_metric m, const U& s1, const rfg_params& p) : CachedScorer(m, s1, p)
    {}
};

} // namespace detail

template <typename CharT1>
struct CachedLevenshtein : detail::CachedIntScorer {
    template <typename Sentence1>
    explicit CachedLevenshtein(const Sentence1& s1, LevenshteinWeightTable w = {1, 1, 1})
        : CachedIntScorer(RFG_LEVENSHTEIN, detail::units(s1), detail::lev_params(w))
    {}
    template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>
    CachedLevenshtein(InputIt1 first1, InputIt1 last1, LevenshteinWeightTable w = {1, 1, 1})
        : CachedIntScorer(RFG_LEVENSHTEIN, detail::units(first1, last1), detail::lev_params(w))
    {}
};

#define RFG_CACHED_INT(NAME, METRIC)                                                                           \
    template <typename CharT1>                                                                                 \
    struct NAME : detail::CachedIntScorer {                                                                    \
        template <typename Sentence1>                                                                          \
        explicit NAME(const Sentence1& s1) : CachedIntScorer(METRIC, detail::units(s1), rfg_params{1, 1, 1, 0.1}) \
        {}                                                                                                     \
        template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>                           \
        NAME(InputIt1 first1, InputIt1 last1)                                                                  \
            : CachedIntScorer(METRIC, detail::units(first1, last1), rfg_params{1, 1, 1, 0.1})                  \
        {}                                                                                                     \
    };
RFG_CACHED_INT(CachedIndel, RFG_INDEL)
RFG_CACHED_INT(CachedLCSseq, RFG_LCSSEQ)
RFG_CACHED_INT(CachedOSA, RFG_OSA)
#undef RFG_CACHED_INT

template <typename CharT1>
struct CachedJaro : detail::CachedDblScorer {
    template <typename Sentence1>
    explicit CachedJaro(const Sentence1& s1) : CachedDblScorer(RFG_JARO, detail::units(s1), rfg_params{1, 1, 1, 0.1})
    {}
    template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>
    CachedJaro(InputIt1 first1, InputIt1 last1)
        : CachedDblScorer(RFG_JARO, detail::units(first1, last1), rfg_params{1, 1, 1, 0.1})
    {}
};

template <typename CharT1>
struct CachedJaroWinkler : detail::CachedDblScorer {
    template <typename Sentence1>
    explicit CachedJaroWinkler(const Sentence1& s1, double prefix_weight = 0.1)
        : CachedDblScorer(RFG_JARO_WINKLER, detail::units(s1), detail::jw_params(prefix_weight))
    {}
    template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>
    CachedJaroWinkler(InputIt1 first1, InputIt1 last1, double prefix_weight = 0.1)
        : CachedDblScorer(RFG_JARO_WINKLER, detail::units(first1, last1), detail::jw_params(prefix_weight))
    {}
};

#if __cplusplus >= 201703L
/* C++17 deduction guides, as in the reference */
template <typename Sentence1>
explicit CachedLevenshtein(const Sentence1&, LevenshteinWeightTable = {1, 1, 1})
    -> CachedLevenshtein<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedIndel(const Sentence1&) -> CachedIndel<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedLCSseq(const Sentence1&) -> CachedLCSseq<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedOSA(const Sentence1&) -> CachedOSA<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedJaro(const Sentence1&) -> CachedJaro<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedJaroWinkler(const Sentence1&, double = 0.1)
    -> CachedJaroWinkler<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
#endif

/* ------------------------------------------------------------------ editops */

/* rapidfuzz/details/types.hpp:28-56 */
enum class EditType { None = 0, Replace = 1, Insert = 2, Delete = 3 };

struct EditOp {
    EditType type = EditType::None;
    size_t src_pos = 0;
    size_t dest_pos = 0;
    EditOp() = default;
    EditOp(EditType t, size_t s, size_t d) : type(t), src_pos(s), dest_pos(d) {}
    bool operator==(const EditOp& o) const { return type == o.type && src_pos == o.src_pos && dest_pos == o.dest_pos; }
    bool operator!=(const EditOp& o) const { return !(*this == o); }
};

namespace detail {
/* the positions a slice takes (details/types.hpp:109-161): a positive step; negative
 * bounds count from the end and clamp at 0, bounds past the end clamp to the size */
inline std::vector<size_t> slice_positions(size_t size, int start, int stop, int step)
{
    if (step == 0) throw std::invalid_argument("slice step cannot be zero");
    if (step < 0) throw std::invalid_argument("step sizes below 0 lead to an invalid order of editops");
    const int n = (int)size;
    start = start < 0 ? std::max(start + n, 0) : std::min(start, n);
    stop = stop < 0 ? std::max(stop + n, 0) : std::min(stop, n);
    std::vector<size_t> pos;
    for (int i = start; i < stop; i += step) pos.push_back((size_t)i);
    return pos;
}
inline EditType swapped(EditType t)
{
    return t == EditType::Insert ? EditType::Delete : t == EditType::Delete ? EditType::Insert : t;
}
} // namespace detail

/* the operations plus the source and destination lengths (details/types.hpp:167-356) */
class Editops : public std::vector<EditOp> {
public:
    Editops() = default;
    size_t get_src_len() const { return src_len_; }
    size_t get_dest_len() const { return dest_len_; }
    void set_src_len(size_t n) { src_len_ = n; }
    void set_dest_len(size_t n) { dest_len_ = n; }

    Editops slice(int start, int stop, int step = 1) const
    {
        Editops r = empty_like();
        for (size_t i : detail::slice_positions(size(), start, stop, step)) r.push_back((*this)[i]);
        return r;
    }
    void remove_slice(int start, int stop, int step = 1)
    {
        const std::vector<size_t> drop = detail::slice_positions(size(), start, stop, step);
        std::vector<EditOp> keep;
        size_t d = 0;
        for (size_t i = 0; i < size(); ++i) {
            if (d < drop.size() && drop[d] == i) ++d;
            else keep.push_back((*this)[i]);
        }
        std::vector<EditOp>::operator=(keep);
    }
    Editops reverse() const
    {
        Editops r(*this);
        std::reverse(r.begin(), r.end());
        return r;
    }
    /* the operations turning the destination into the source */
    Editops inverse() const
    {
        Editops r;
        r.src_len_ = dest_len_;
        r.dest_len_ = src_len_;
        for (const EditOp& op : *this) r.emplace_back(detail::swapped(op.type), op.dest_pos, op.src_pos);
        return r;
    }
    /* the operations left once those of sub (in order) are taken out; source positions
     * shift by the removed insertions and deletions */
    Editops remove_subsequence(const Editops& sub) const
    {
        if (sub.size() > size()) throw std::invalid_argument("subsequence is not a subsequence");
        Editops r = empty_like();
        long long offset = 0;
        size_t it = 0;
        auto keep = [&](const EditOp& op) {
            r.emplace_back(op.type, (size_t)((long long)op.src_pos + offset), op.dest_pos);
        };
        for (const EditOp& sop : sub) {
            for (; it < size() && (*this)[it] != sop; ++it) keep((*this)[it]);
            if (it == size()) throw std::invalid_argument("subsequence is not a subsequence");
            offset += sop.type == EditType::Insert ? 1 : sop.type == EditType::Delete ? -1 : 0;
            ++it;
        }
        for (; it < size(); ++it) keep((*this)[it]);
        return r;
    }

private:
    Editops empty_like() const
    {
        Editops r;
        r.src_len_ = src_len_;
        r.dest_len_ = dest_len_;
        return r;
    }
    size_t src_len_ = 0, dest_len_ = 0;
};

namespace detail {
template <typename U1, typename U2>
Editops editops(rfg_metric m, const U1& a, const U2& b, size_t score_hint)
{
    int64_t o1[2] = {0, a.len}, o2[2] = {0, b.len};
    rfg_strings s1{a.data, o1, 1, a.width}, s2{b.data, o2, 1, b.width};
    std::vector<rfg_editop> ops((size_t)(a.len + b.len) + 1);
    int64_t off[2] = {0, 0};
    throw_on(rfg_editops(m, &s1, &s2, (uint64_t)score_hint, ops.data(), (int64_t)ops.size(), off, 0));
    Editops e;
    for (int64_t k = off[0]; k < off[1]; ++k)
        e.emplace_back((EditType)ops[(size_t)k].type, (size_t)ops[(size_t)k].src_pos, (size_t)ops[(size_t)k].dest_pos);
    e.set_src_len((size_t)a.len);
    e.set_dest_len((size_t)b.len);
    return e;
}
} // namespace detail

/* runs of operations (details/types.hpp:81-100): None runs are the unchanged stretches */
struct Opcode {
    EditType type = EditType::None;
    size_t src_begin = 0, src_end = 0, dest_begin = 0, dest_end = 0;
    Opcode() = default;
    Opcode(EditType t, size_t sb, size_t se, size_t db, size_t de)
        : type(t), src_begin(sb), src_end(se), dest_begin(db), dest_end(de)
    {}
    bool operator==(const Opcode& o) const
    {
        return type == o.type && src_begin == o.src_begin && src_end == o.src_end && dest_begin == o.dest_begin &&
               dest_end == o.dest_end;
    }
};

/* Opcodes(const Editops&) (details/types.hpp:526-569): gaps between operations become None
 * runs, consecutive operations of one type that continue each other merge into one run */
class Opcodes : public std::vector<Opcode> {
public:
    Opcodes() = default;
    explicit Opcodes(const Editops& e) : src_len_(e.get_src_len()), dest_len_(e.get_dest_len())
    {
        size_t sp = 0, dp = 0;
        for (size_t i = 0; i < e.size();) {
            if (sp < e[i].src_pos || dp < e[i].dest_pos) {
                emplace_back(EditType::None, sp, e[i].src_pos, dp, e[i].dest_pos);
                sp = e[i].src_pos;
                dp = e[i].dest_pos;
            }
            const size_t sb = sp, db = dp;
            const EditType t = e[i].type;
            do {
                sp += (t == EditType::Replace || t == EditType::Delete);
                dp += (t == EditType::Replace || t == EditType::Insert);
                ++i;
            } while (i < e.size() && e[i].type == t && e[i].src_pos == sp && e[i].dest_pos == dp);
            emplace_back(t, sb, sp, db, dp);
        }
        if (sp < src_len_ || dp < dest_len_) emplace_back(EditType::None, sp, src_len_, dp, dest_len_);
    }
    size_t get_src_len() const { return src_len_; }
    size_t get_dest_len() const { return dest_len_; }
    Opcodes slice(int start, int stop, int step = 1) const
    {
        Opcodes r = empty_like();
        for (size_t i : detail::slice_positions(size(), start, stop, step)) r.push_back((*this)[i]);
        return r;
    }
    Opcodes reverse() const
    {
        Opcodes r(*this);
        std::reverse(r.begin(), r.end());
        return r;
    }
    Opcodes inverse() const
    {
        Opcodes r;
        r.src_len_ = dest_len_;
        r.dest_len_ = src_len_;
        for (const Opcode& o : *this)
            r.emplace_back(detail::swapped(o.type), o.dest_begin, o.dest_end, o.src_begin, o.src_end);
        return r;
    }
    /* Editops(const Opcodes&) (details/types.hpp:500-524) */
    Editops as_editops() const
    {
        Editops e;
        e.set_src_len(src_len_);
        e.set_dest_len(dest_len_);
        for (const Opcode& o : *this) {
            if (o.type == EditType::Replace)
                for (size_t j = 0; j < o.src_end - o.src_begin; ++j)
                    e.emplace_back(EditType::Replace, o.src_begin + j, o.dest_begin + j);
            else if (o.type == EditType::Insert)
                for (size_t j = 0; j < o.dest_end - o.dest_begin; ++j)
                    e.emplace_back(EditType::Insert, o.src_begin, o.dest_begin + j);
            else if (o.type == EditType::Delete)
                for (size_t j = 0; j < o.src_end - o.src_begin; ++j)
                    e.emplace_back(EditType::Delete, o.src_begin + j, o.dest_begin);
        }
        return e;
    }

private:
    Opcodes empty_like() const
    {
        Opcodes r;
        r.src_len_ = src_len_;
        r.dest_len_ = dest_len_;
        return r;
    }
    size_t src_len_ = 0, dest_len_ = 0;
};

/* editops_apply_* / opcodes_apply_* (rapidfuzz/distance.hpp:19-160): s1 turned into s2 */
template <typename CharT, typename Sentence1, typename Sentence2>
std::vector<CharT> editops_apply_vec(const Editops& ops, const Sentence1& s1, const Sentence2& s2)
{
    std::vector<CharT> r;
    size_t sp = 0;
    for (const EditOp& op : ops) {
        for (; sp < op.src_pos; ++sp) r.push_back((CharT)s1[sp]);
        if (op.type == EditType::None || op.type == EditType::Replace) {
            r.push_back((CharT)s2[op.dest_pos]);
            ++sp;
        }
        else if (op.type == EditType::Insert) r.push_back((CharT)s2[op.dest_pos]);
        else ++sp;
    }
    for (; sp < (size_t)std::distance(std::begin(s1), std::end(s1)); ++sp) r.push_back((CharT)s1[sp]);
    return r;
}
template <typename CharT, typename Sentence1, typename Sentence2>
std::basic_string<CharT> editops_apply_str(const Editops& ops, const Sentence1& s1, const Sentence2& s2)
{
    const std::vector<CharT> v = editops_apply_vec<CharT>(ops, s1, s2);
    return std::basic_string<CharT>(v.begin(), v.end());
}
template <typename CharT, typename Sentence1, typename Sentence2>
std::vector<CharT> opcodes_apply_vec(const Opcodes& ops, const Sentence1& s1, const Sentence2& s2)
{
    std::vector<CharT> r;
    for (const Opcode& o : ops) {
        if (o.type == EditType::None)
            for (size_t i = o.src_begin; i < o.src_end; ++i) r.push_back((CharT)s1[i]);
        else if (o.type != EditType::Delete)
            for (size_t i = o.dest_begin; i < o.dest_end; ++i) r.push_back((CharT)s2[i]);
    }
    return r;
}
template <typename CharT, typename Sentence1, typename Sentence2>
std::basic_string<CharT> opcodes_apply_str(const Opcodes& ops, const Sentence1& s1, const Sentence2& s2)
{
    const std::vector<CharT> v = opcodes_apply_vec<CharT>(ops, s1, s2);
    return std::basic_string<CharT>(v.begin(), v.end());
}

/* Levenshtein.hpp:282-295 */
template <typename Sentence1, typename Sentence2>
Editops levenshtein_editops(const Sentence1& s1, const Sentence2& s2,
                            size_t score_hint = std::numeric_limits<size_t>::max())
{
    return detail::editops(RFG_LEVENSHTEIN, detail::units(s1), detail::units(s2), score_hint);
}
template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>
Editops levenshtein_editops(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2,
                            size_t score_hint = std::numeric_limits<size_t>::max())
{
    return detail::editops(RFG_LEVENSHTEIN, detail::units(first1, last1), detail::units(first2, last2), score_hint);
}

/* Indel.hpp:65-75, LCSseq.hpp:65-75 */
template <typename Sentence1, typename Sentence2>
Editops indel_editops(const Sentence1& s1, const Sentence2& s2)
{
    return detail::editops(RFG_INDEL, detail::units(s1), detail::units(s2), 0);
}
template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>
Editops indel_editops(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2)
{
    return detail::editops(RFG_INDEL, detail::units(first1, last1), detail::units(first2, last2), 0);
}
template <typename Sentence1, typename Sentence2>
Editops lcs_seq_editops(const Sentence1& s1, const Sentence2& s2)
{
    return detail::editops(RFG_LCSSEQ, detail::units(s1), detail::units(s2), 0);
}
template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>
Editops lcs_seq_editops(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2)
{
    return detail::editops(RFG_LCSSEQ, detail::units(first1, last1), detail::units(first2, last2), 0);
}

/* --------------------------------------------------------------------- fuzz */

namespace fuzz {

/* fuzz.hpp:44-48 */
template <typename Sentence1, typename Sentence2>
double ratio(const Sentence1& s1, const Sentence2& s2, double score_cutoff = 0)
{
    return detail::score_f(RFG_RATIO, RFG_SIMILARITY, detail::units(s1), detail::units(s2), rfg_params{1, 1, 1, 0.1},
                           score_cutoff, score_cutoff);
}
template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>
double ratio(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2, double score_cutoff = 0)
{
    return detail::score_f(RFG_RATIO, RFG_SIMILARITY, detail::units(first1, last1), detail::units(first2, last2),
                           rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);
}

/* fuzz.hpp:99-126 */
template <typename CharT1>
struct CachedRatio : rapidfuzz_gb300::detail::CachedScorer {
    template <typename Sentence1>
    CachedRatio(const Sentence1& s1)
        : CachedScorer(RFG_RATIO, rapidfuzz_gb300::detail::units(s1), rfg_params{1, 1, 1, 0.1})
    {}
    template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>
    CachedRatio(InputIt1 first1, InputIt1 last1)
        : CachedScorer(RFG_RATIO, rapidfuzz_gb300::detail::units(first1, last1), rfg_params{1, 1, 1, 0.1})
    {}
    template <typename Sentence2>
    double similarity(const Sentence2& s2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_SIMILARITY, rapidfuzz_gb300::detail::units(s2), score_cutoff, score_hint);
    }
    template <typename InputIt2, rapidfuzz_gb300::detail::if_iter<InputIt2> = 0>
    double similarity(InputIt2 first2, InputIt2 last2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_SIMILARITY, rapidfuzz_gb300::detail::units(first2, last2), score_cutoff, score_hint);
    }
};

/* fuzz.hpp:128-147 (partial_ratio, fuzz_impl.hpp:194-239) */
template <typename Sentence1, typename Sentence2>
double partial_ratio(const Sentence1& s1, const Sentence2& s2, double score_cutoff = 0)
{
    return detail::score_f(RFG_PARTIAL_RATIO, RFG_SIMILARITY, detail::units(s1), detail::units(s2),
                           rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);
}
template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>
double partial_ratio(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2, double score_cutoff = 0)
{
    return detail::score_f(RFG_PARTIAL_RATIO, RFG_SIMILARITY, detail::units(first1, last1),
                           detail::units(first2, last2), rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);
}

/* fuzz.hpp:158-183 (CachedPartialRatio, fuzz_impl.hpp:241-283) */
template <typename CharT1>
struct CachedPartialRatio : rapidfuzz_gb300::detail::CachedScorer {
    template <typename Sentence1>
    CachedPartialRatio(const Sentence1& s1)
        : CachedScorer(RFG_PARTIAL_RATIO, rapidfuzz_gb300::detail::units(s1), rfg_params{1, 1, 1, 0.1})
    {}
    template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>
    CachedPartialRatio(InputIt1 first1, InputIt1 last1)
        : CachedScorer(RFG_PARTIAL_RATIO, rapidfuzz_gb300::detail::units(first1, last1), rfg_params{1, 1, 1, 0.1})
    {}
    template <typename Sentence2>
    double similarity(const Sentence2& s2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_SIMILARITY, rapidfuzz_gb300::detail::units(s2), score_cutoff, score_hint);
    }
    template <typename InputIt2, rapidfuzz_gb300::detail::if_iter<InputIt2> = 0>
    double similarity(InputIt2 first2, InputIt2 last2, double score_cutoff = 0.0, double score_hint = 0.0) const
    {
        return cached_f(RFG_SIMILARITY, rapidfuzz_gb300::detail::units(first2, last2), score_cutoff, score_hint);
    }
};

/* token_sort_ratio (fuzz.hpp:203-234, fuzz_impl.hpp:297-311), partial_token_sort_ratio
 * (fuzz.hpp:313-341, fuzz_impl.hpp:334-349), QRatio (fuzz.hpp:692-717,
 * fuzz_impl.hpp:891-909).  Tokens compare as unsigned code units (for `char` strings this
 * is the reference's order where `char` is unsigned). */
#define RFG_FUZZ_FREE(NAME, METRIC)                                                                                \
    template <typename Sentence1, typename Sentence2>                                                              \
    double NAME(const Sentence1& s1, const Sentence2& s2, double score_cutoff = 0)                                 \
    {                                                                                                              \
        return detail::score_f(METRIC, RFG_SIMILARITY, detail::units(s1), detail::units(s2),                       \
                               rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);                              \
    }                                                                                                              \
    template <typename InputIt1, typename InputIt2, detail::if_iter<InputIt1> = 0>                                 \
    double NAME(InputIt1 first1, InputIt1 last1, InputIt2 first2, InputIt2 last2, double score_cutoff = 0)         \
    {                                                                                                              \
        return detail::score_f(METRIC, RFG_SIMILARITY, detail::units(first1, last1), detail::units(first2, last2), \
                               rfg_params{1, 1, 1, 0.1}, score_cutoff, score_cutoff);                              \
    }
RFG_FUZZ_FREE(token_sort_ratio, RFG_TOKEN_SORT_RATIO)
RFG_FUZZ_FREE(partial_token_sort_ratio, RFG_PARTIAL_TOKEN_SORT_RATIO)
RFG_FUZZ_FREE(QRatio, RFG_QRATIO)
/* fuzz.hpp:375-690: token_set_ratio, partial_token_set_ratio, token_ratio,
 * partial_token_ratio, WRatio */
RFG_FUZZ_FREE(token_set_ratio, RFG_TOKEN_SET_RATIO)
RFG_FUZZ_FREE(partial_token_set_ratio, RFG_PARTIAL_TOKEN_SET_RATIO)
RFG_FUZZ_FREE(token_ratio, RFG_TOKEN_RATIO)
RFG_FUZZ_FREE(partial_token_ratio, RFG_PARTIAL_TOKEN_RATIO)
RFG_FUZZ_FREE(WRatio, RFG_WRATIO)
#undef RFG_FUZZ_FREE

/* CachedTokenSortRatio (fuzz.hpp:282-305), CachedPartialTokenSortRatio (fuzz.hpp:342-366),
 * CachedQRatio (fuzz.hpp:776-797): s1 (its sorted-split join for the token sorts) lives
 * on the device */
#define RFG_FUZZ_CACHED(NAME, METRIC)                                                                              \
    template <typename CharT1>                                                                                     \
    struct NAME : rapidfuzz_gb300::detail::CachedScorer {                                                          \
        template <typename Sentence1>                                                                              \
        explicit NAME(const Sentence1& s1)                                                                         \
            : CachedScorer(METRIC, rapidfuzz_gb300::detail::units(s1), rfg_params{1, 1, 1, 0.1})                   \
        {}                                                                                                         \
        template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>                              \
        NAME(InputIt1 first1, InputIt1 last1)                                                                      \
            : CachedScorer(METRIC, rapidfuzz_gb300::detail::units(first1, last1), rfg_params{1, 1, 1, 0.1})        \
        {}                                                                                                         \
        template <typename Sentence2>                                                                              \
        double similarity(const Sentence2& s2, double score_cutoff = 0.0, double score_hint = 0.0) const           \
        {                                                                                                          \
            return cached_f(RFG_SIMILARITY, rapidfuzz_gb300::detail::units(s2), score_cutoff, score_hint);         \
        }                                                                                                          \
        template <typename InputIt2, rapidfuzz_gb300::detail::if_iter<InputIt2> = 0>                              \
        double similarity(InputIt2 first2, InputIt2 last2, double score_cutoff = 0.0,                              \
                          double score_hint = 0.0) const                                                           \
        {                                                                                                          \
            return cached_f(RFG_SIMILARITY, rapidfuzz_gb300::detail::units(first2, last2), score_cutoff,           \
                            score_hint);                                                                           \
        }                                                                                                          \
    };
RFG_FUZZ_CACHED(CachedTokenSortRatio, RFG_TOKEN_SORT_RATIO)
RFG_FUZZ_CACHED(CachedPartialTokenSortRatio, RFG_PARTIAL_TOKEN_SORT_RATIO)
RFG_FUZZ_CACHED(CachedQRatio, RFG_QRATIO)
RFG_FUZZ_CACHED(CachedTokenSetRatio, RFG_TOKEN_SET_RATIO)
RFG_FUZZ_CACHED(CachedPartialTokenSetRatio, RFG_PARTIAL_TOKEN_SET_RATIO)
RFG_FUZZ_CACHED(CachedTokenRatio, RFG_TOKEN_RATIO)
RFG_FUZZ_CACHED(CachedPartialTokenRatio, RFG_PARTIAL_TOKEN_RATIO)
RFG_FUZZ_CACHED(CachedWRatio, RFG_WRATIO)
#undef RFG_FUZZ_CACHED

#if __cplusplus >= 201703L
template <typename Sentence1>
explicit CachedTokenSortRatio(const Sentence1&)
    -> CachedTokenSortRatio<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedPartialTokenSortRatio(const Sentence1&)
    -> CachedPartialTokenSortRatio<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
template <typename Sentence1>
explicit CachedQRatio(const Sentence1&)
    -> CachedQRatio<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
#define RFG_FUZZ_GUIDE(NAME)                                                                                       \
    template <typename Sentence1>                                                                                  \
    explicit NAME(const Sentence1&)->NAME<typename std::decay<decltype(*std::begin(std::declval<Sentence1>()))>::type>;
RFG_FUZZ_GUIDE(CachedTokenSetRatio)
RFG_FUZZ_GUIDE(CachedPartialTokenSetRatio)
RFG_FUZZ_GUIDE(CachedTokenRatio)
RFG_FUZZ_GUIDE(CachedPartialTokenRatio)
RFG_FUZZ_GUIDE(CachedWRatio)
#undef RFG_FUZZ_GUIDE
#endif

} // namespace fuzz

/* ---------------------------------------------------------------- Multi* */

namespace experimental {

namespace detail_multi {

template <rfg_metric M, int MaxLen, bool IntResult>
class MultiScorer {
public:
    static_assert(MaxLen == 8 || MaxLen == 16 || MaxLen == 32 || MaxLen == 64, "expected MaxLen in 8/16/32/64");
    MultiScorer(const MultiScorer&) = delete;
    MultiScorer& operator=(const MultiScorer&) = delete;
    ~MultiScorer()
    {
        if (h_) rfg_multi_destroy(h_);
    }
    size_t result_count() const
    {
        size_t n = 0;
        rapidfuzz_gb300::detail::throw_on(rfg_multi_result_count(h_, &n));
        return n;
    }
    template <typename Sentence1>
    void insert(const Sentence1& s1)
    {
        auto u = rapidfuzz_gb300::detail::units(s1);
        rapidfuzz_gb300::detail::throw_on(rfg_multi_insert(h_, u.data, u.len, u.width));
    }
    template <typename InputIt1, rapidfuzz_gb300::detail::if_iter<InputIt1> = 0>
    void insert(InputIt1 first1, InputIt1 last1)
    {
        auto u = rapidfuzz_gb300::detail::units(first1, last1);
        rapidfuzz_gb300::detail::throw_on(rfg_multi_insert(h_, u.data, u.len, u.width));
    }

protected:
    MultiScorer(size_t count, const rfg_params& p)
    {
        rapidfuzz_gb300::detail::throw_on(rfg_multi_create(M, MaxLen, count, &p, &h_));
    }
    template <typename Sentence2>
    void run_i(rfg_op op, size_t* scores, size_t n, const Sentence2& s2, size_t cutoff) const
    {
        static_assert(sizeof(size_t) == sizeof(int64_t), "64-bit size_t expected");
        auto u = rapidfuzz_gb300::detail::units(s2);
        rapidfuzz_gb300::detail::throw_on(
            rfg_multi_score_i64(h_, op, reinterpret_cast<int64_t*>(scores), n, u.data, u.len, u.width, cutoff));
    }
    template <typename Sentence2>
    void run_f(rfg_op op, double* scores, size_t n, const Sentence2& s2, double cutoff) const
    {
        auto u = rapidfuzz_gb300::detail::units(s2);
        rapidfuzz_gb300::detail::throw_on(rfg_multi_score_f64(h_, op, scores, n, u.data, u.len, u.width, cutoff));
    }
    rfg_multi h_ = nullptr;
};

/* MultiDistanceBase / MultiSimilarityBase (distance.hpp:390-582) over size_t scores */
template <rfg_metric M, int MaxLen>
class MultiIntScorer : public MultiScorer<M, MaxLen, true> {
public:
    template <typename Sentence2>
    void distance(size_t* scores, size_t score_count, const Sentence2& s2,
                  size_t score_cutoff = (size_t)std::numeric_limits<int64_t>::max()) const
    {
        this->run_i(RFG_DISTANCE, scores, score_count, s2, score_cutoff);
    }
    template <typename Sentence2>
    void similarity(size_t* scores, size_t score_count, const Sentence2& s2, size_t score_cutoff = 0) const
    {
        this->run_i(RFG_SIMILARITY, scores, score_count, s2, score_cutoff);
    }
    template <typename Sentence2>
    void normalized_distance(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 1.0) const
    {
        this->run_f(RFG_NORMALIZED_DISTANCE, scores, score_count, s2, score_cutoff);
    }
    template <typename Sentence2>
    void normalized_similarity(double* scores, size_t score_count, const Sentence2& s2,
                               double score_cutoff = 0.0) const
    {
        this->run_f(RFG_NORMALIZED_SIMILARITY, scores, score_count, s2, score_cutoff);
    }

protected:
    MultiIntScorer(size_t count, const rfg_params& p) : MultiScorer<M, MaxLen, true>(count, p)
    {}
};

template <rfg_metric M, int MaxLen>
class MultiDblScorer : public MultiScorer<M, MaxLen, false> {
public:
    template <typename Sentence2>
    void distance(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 1.0) const
    {
        this->run_f(RFG_DISTANCE, scores, score_count, s2, score_cutoff);
    }
    template <typename Sentence2>
    void similarity(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 0.0) const
    {
        this->run_f(RFG_SIMILARITY, scores, score_count, s2, score_cutoff);
    }
    template <typename Sentence2>
    void normalized_distance(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 1.0) const
    {
        this->run_f(RFG_NORMALIZED_DISTANCE, scores, score_count, s2, score_cutoff);
    }
    template <typename Sentence2>
    void normalized_similarity(double* scores, size_t score_count, const Sentence2& s2,
                               double score_cutoff = 0.0) const
    {
        this->run_f(RFG_NORMALIZED_SIMILARITY, scores, score_count, s2, score_cutoff);
    }

protected:
    MultiDblScorer(size_t count, const rfg_params& p) : MultiScorer<M, MaxLen, false>(count, p)
    {}
};

} // namespace detail_multi

template <int MaxLen>
struct MultiLevenshtein : detail_multi::MultiIntScorer<RFG_LEVENSHTEIN, MaxLen> {
    MultiLevenshtein(size_t count, LevenshteinWeightTable w = {1, 1, 1})
        : detail_multi::MultiIntScorer<RFG_LEVENSHTEIN, MaxLen>(count, rapidfuzz_gb300::detail::lev_params(w))
    {}
};
template <int MaxLen>
struct MultiIndel : detail_multi::MultiIntScorer<RFG_INDEL, MaxLen> {
    MultiIndel(size_t count) : detail_multi::MultiIntScorer<RFG_INDEL, MaxLen>(count, rfg_params{1, 1, 1, 0.1})
    {}
};
template <int MaxLen>
struct MultiLCSseq : detail_multi::MultiIntScorer<RFG_LCSSEQ, MaxLen> {
    MultiLCSseq(size_t count) : detail_multi::MultiIntScorer<RFG_LCSSEQ, MaxLen>(count, rfg_params{1, 1, 1, 0.1})
    {}
};
template <int MaxLen>
struct MultiOSA : detail_multi::MultiIntScorer<RFG_OSA, MaxLen> {
    MultiOSA(size_t count) : detail_multi::MultiIntScorer<RFG_OSA, MaxLen>(count, rfg_params{1, 1, 1, 0.1})
    {}
};
template <int MaxLen>
struct MultiJaro : detail_multi::MultiDblScorer<RFG_JARO, MaxLen> {
    MultiJaro(size_t count) : detail_multi::MultiDblScorer<RFG_JARO, MaxLen>(count, rfg_params{1, 1, 1, 0.1})
    {}
};
template <int MaxLen>
struct MultiJaroWinkler : detail_multi::MultiDblScorer<RFG_JARO_WINKLER, MaxLen> {
    MultiJaroWinkler(size_t count, double prefix_weight = 0.1)
        : detail_multi::MultiDblScorer<RFG_JARO_WINKLER, MaxLen>(count, rapidfuzz_gb300::detail::jw_params(prefix_weight))
    {}
};

} // namespace experimental

namespace fuzz {
namespace experimental {
/* fuzz.hpp:50-95 */
template <int MaxLen>
struct MultiRatio : rapidfuzz_gb300::experimental::detail_multi::MultiScorer<RFG_RATIO, MaxLen, false> {
    MultiRatio(size_t count)
        : rapidfuzz_gb300::experimental::detail_multi::MultiScorer<RFG_RATIO, MaxLen, false>(count,
                                                                                           rfg_params{1, 1, 1, 0.1})
    {}
    template <typename Sentence2>
    void similarity(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 0) const
    {
        this->run_f(RFG_SIMILARITY, scores, score_count, s2, score_cutoff);
    }
};

/* fuzz.hpp:236-278 (insert keeps the sorted-split join) */
template <int MaxLen>
struct MultiTokenSortRatio
    : rapidfuzz_gb300::experimental::detail_multi::MultiScorer<RFG_TOKEN_SORT_RATIO, MaxLen, false> {
    MultiTokenSortRatio(size_t count)
        : rapidfuzz_gb300::experimental::detail_multi::MultiScorer<RFG_TOKEN_SORT_RATIO, MaxLen, false>(
              count, rfg_params{1, 1, 1, 0.1})
    {}
    template <typename Sentence2>
    void similarity(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 0) const
    {
        this->run_f(RFG_SIMILARITY, scores, score_count, s2, score_cutoff);
    }
};

/* fuzz.hpp:719-774 */
template <int MaxLen>
struct MultiQRatio : rapidfuzz_gb300::experimental::detail_multi::MultiScorer<RFG_QRATIO, MaxLen, false> {
    MultiQRatio(size_t count)
        : rapidfuzz_gb300::experimental::detail_multi::MultiScorer<RFG_QRATIO, MaxLen, false>(count,
                                                                                            rfg_params{1, 1, 1, 0.1})
    {}
    template <typename Sentence2>
    void similarity(double* scores, size_t score_count, const Sentence2& s2, double score_cutoff = 0) const
    {
        this->run_f(RFG_SIMILARITY, scores, score_count, s2, score_cutoff);
    }
};
} // namespace experimental
} // namespace fuzz

} // namespace rapidfuzz_gb300
