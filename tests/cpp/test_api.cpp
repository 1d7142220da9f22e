// C++ drop-in check: the rapidfuzz-cpp API of rapidfuzz_gb300 (GPU through the C ABI)
// against the CPU oracle, with the known answers of the reference's tests
// (test/distance/tests-*.cpp) and a seeded random sweep.  Exit code 0 = pass.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "rapidfuzz_gb300/rapidfuzz.hpp"
#include "rfo.h"

namespace rapidfuzz = rapidfuzz_gb300;

static int failures = 0;
#define CHECK(cond)                                                                                    \
    do {                                                                                               \
        if (!(cond)) {                                                                                 \
            std::printf("FAIL %s:%d: %s\n", __FILE__, __LINE__, #cond);                                \
            ++failures;                                                                                \
        }                                                                                              \
    } while (0)

static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }

static int64_t oi(int m, int op, int form, const std::string& a, const std::string& b, uint64_t c,
                  rfo_params p = {1, 1, 1, 0.1})
{
    int64_t r = 0;
    double f = 0;
    rfo_score(m, op, form, a.data(), (int64_t)a.size(), 1, b.data(), (int64_t)b.size(), 1, &p, c, 0.0, &r, &f);
    return r;
}

static double of(int m, int op, int form, const std::string& a, const std::string& b, double c,
                 rfo_params p = {1, 1, 1, 0.1})
{
    int64_t r = 0;
    double f = 0;
    rfo_score(m, op, form, a.data(), (int64_t)a.size(), 1, b.data(), (int64_t)b.size(), 1, &p, 0, c, &r, &f);
    return f;
}

int main()
{
    using rapidfuzz::LevenshteinWeightTable;
    // tests-Levenshtein.cpp:98-141
    std::string test = "aaaa", no_suffix2 = "aaab", swapped1 = "abaa", swapped2 = "baaa", replace_all = "bbbb";
    std::wstring no_suffix = L"aaa";
    CHECK(rapidfuzz::levenshtein_distance(std::string(""), std::string("")) == 0);
    CHECK(rapidfuzz::levenshtein_distance(test, std::string("")) == 4);
    CHECK(rapidfuzz::levenshtein_distance(test, no_suffix) == 1);
    CHECK(rapidfuzz::levenshtein_distance(swapped1, swapped2) == 2);
    CHECK(rapidfuzz::levenshtein_distance(test, no_suffix2) == 1);
    CHECK(rapidfuzz::levenshtein_distance(test, replace_all) == 4);
    CHECK(rapidfuzz::levenshtein_distance(test, replace_all, {1, 1, 2}) == 8);
    CHECK(rapidfuzz::levenshtein_normalized_similarity(test, test, {1, 1, 2}) == 1.0);
    CHECK(std::fabs(rapidfuzz::levenshtein_normalized_similarity(test, no_suffix, {1, 1, 2}) - 0.8571) < 1e-4);
    CHECK(rapidfuzz::levenshtein_distance("lewenstein", "levenshtein") == 2);
    // tests-Levenshtein.cpp:143-179 (mbleven cutoffs)
    std::string a = "South Korea", b = "North Korea";
    CHECK(rapidfuzz::levenshtein_distance(a, b, {1, 1, 1}, 1) == 2);
    CHECK(rapidfuzz::levenshtein_distance(a, b, {1, 1, 1}, 0) == 1);
    CHECK(rapidfuzz::levenshtein_distance(a, b, {1, 1, 2}, 2) == 3);
    // Cached and iterator forms agree (tests-Levenshtein.cpp:21-96)
    rapidfuzz::CachedLevenshtein<char> scorer(a);
    CHECK(scorer.distance(b) == 2);
    CHECK(scorer.distance(b.begin(), b.end()) == 2);
    CHECK(scorer.similarity(b) == 9);
#if __cplusplus >= 201703L
    rapidfuzz::CachedLevenshtein deduced(a, {1, 1, 2});
    CHECK(deduced.distance(b) == 4);
#endif
    // Indel / LCSseq (tests-Indel.cpp:222-247, tests-LCSseq.cpp:166-196)
    CHECK(rapidfuzz::indel_distance(a, b) == 4);
    CHECK(rapidfuzz::indel_distance(a, b, 2) == 3);
    CHECK(rapidfuzz::lcs_seq_similarity(a, b) == 9);
    CHECK(rapidfuzz::lcs_seq_similarity(a, b, 10) == 0);
    rapidfuzz::CachedIndel<char> ci(std::string("001"));
    CHECK(std::fabs(ci.normalized_similarity(std::string("220")) - 0.3333333) < 1e-6);
    // OSA (tests-OSA.cpp:59-96)
    CHECK(rapidfuzz::osa_distance(std::string("CA"), std::string("AC")) == 1);
    CHECK(rapidfuzz::osa_distance(std::string("CA"), std::string("ABC")) == 3);
    std::string filler(64, 'a');
    CHECK(rapidfuzz::osa_distance("a" + filler + "CA" + filler + "a", "b" + filler + "AC" + filler + "b") == 3);
    // Jaro / JW (tests-Jaro.cpp:172-178, tests-JaroWinkler.cpp:177-183)
    CHECK(std::fabs(rapidfuzz::jaro_similarity(std::string("0"), std::string("00")) - 0.833333) < 1e-6);
    CHECK(std::fabs(rapidfuzz::jaro_winkler_similarity(std::string("0"), std::string("00")) - 0.85) < 1e-6);
    rapidfuzz::CachedJaroWinkler<char> jw(std::string("000000001"));
    CHECK(std::fabs(jw.similarity(std::string("0000010")) - 0.926984127) < 1e-6);
    // fuzz::ratio (tests-fuzz.cpp:52-60)
    CHECK(std::fabs(rapidfuzz::fuzz::ratio(std::string("new york mets"), std::string("new york mets")) - 100) < 1e-6);
    rapidfuzz::fuzz::CachedRatio<char> cr(std::string("new york mets"));
    CHECK(std::fabs(cr.similarity(std::string("the wonderful new york mets")) - 65) < 1);
    // fuzz::partial_ratio (tests-fuzz.cpp:154-158)
    CHECK(std::fabs(rapidfuzz::fuzz::partial_ratio(std::string("001"), std::string("220222")) - 33.3333333) < 1e-6);
    rapidfuzz::fuzz::CachedPartialRatio<char> cpr(std::string("physics 2 vid"));
    CHECK(cpr.similarity(std::string("study physics physics 2 video")) == 100.0);
    // token scorers (tests-fuzz.cpp:82-86, 127-137)
    CHECK(rapidfuzz::fuzz::token_sort_ratio(std::string("new york mets"), std::string("new york mets")) == 100.0);
    CHECK(rapidfuzz::fuzz::token_sort_ratio(std::string("new york mets vs atlanta braves"),
                                            std::string("atlanta braves vs new york mets")) == 100.0);
    CHECK(rapidfuzz::fuzz::token_sort_ratio(std::string(""), std::string("")) == 100.0);
    CHECK(rapidfuzz::fuzz::partial_token_sort_ratio(std::string(""), std::string("")) == 100.0);
    CHECK(rapidfuzz::fuzz::QRatio(std::string(""), std::string("")) == 0.0);
    CHECK(rapidfuzz::fuzz::QRatio(std::string("new york mets"), std::string("new york mets")) == 100.0);
    rapidfuzz::fuzz::CachedTokenSortRatio<char> cts(std::string("mets new york"));
    CHECK(cts.similarity(std::string("york  mets\tnew")) == 100.0);
    rapidfuzz::fuzz::CachedPartialTokenSortRatio<char> cpts(std::string("york new"));
    CHECK(cpts.similarity(std::string("mets new york")) == 100.0);
    rapidfuzz::fuzz::CachedQRatio<char> cq(std::string(""));
    CHECK(cq.similarity(std::string("")) == 0.0);
    {
        rapidfuzz::fuzz::experimental::MultiTokenSortRatio<16> mts(2);
        mts.insert(std::string("  b a  "));
        mts.insert(std::string("  c     b   a        "));  // 21 units; MaxLen applies to the join "a b c"
        std::vector<double> r(mts.result_count());
        mts.similarity(r.data(), r.size(), std::string("a b"));
        CHECK(r[0] == 100.0 && r[1] == 75.0);
    }
    {
        rapidfuzz::fuzz::experimental::MultiQRatio<8> mq(2);
        mq.insert(std::string(""));
        mq.insert(std::string("ab"));
        std::vector<double> r(mq.result_count(), -1.0);
        mq.similarity(r.data(), r.size(), std::string("ab"));
        CHECK(r[0] == 0.0 && r[1] == 100.0);
        mq.similarity(r.data(), r.size(), std::string(""));
        CHECK(r[0] == 0.0 && r[1] == 0.0);
    }
    // editops (tests-Levenshtein.cpp:235-244): applying the operations turns s into d
    {
        const std::string s = "Lorem ipsum.", d = "XYZLorem ABC iPsum";
        rapidfuzz::Editops ops = rapidfuzz::levenshtein_editops(s, d);
        CHECK(ops.get_src_len() == s.size() && ops.get_dest_len() == d.size());
        std::string r;
        size_t sp = 0;
        for (const auto& op : ops) { /* apply in order (editops_apply_str, distance.hpp:19-60) */
            while (sp < op.src_pos) r += s[sp++];
            if (op.type == rapidfuzz::EditType::Insert) r += d[op.dest_pos];
            else if (op.type == rapidfuzz::EditType::Replace) { r += d[op.dest_pos]; ++sp; }
            else if (op.type == rapidfuzz::EditType::Delete) ++sp;
        }
        while (sp < s.size()) r += s[sp++];
        CHECK(r == d);
        CHECK(rapidfuzz::editops_apply_str<char>(ops, s, d) == d);
        rapidfuzz::Opcodes oc(ops);
        CHECK(rapidfuzz::opcodes_apply_str<char>(oc, s, d) == d);
        CHECK(oc.as_editops() == ops);
        CHECK(oc.get_src_len() == s.size() && oc.get_dest_len() == d.size());
        CHECK(rapidfuzz::indel_editops(std::string("kitten"), std::string("sitting")).size() == 5);
        CHECK(rapidfuzz::lcs_seq_editops(std::string("kitten"), std::string("sitting")).size() == 5);
        CHECK(rapidfuzz::levenshtein_editops(std::string("kitten"), std::string("sitting")).size() == 3);
    }
    // token_set_ratio family (tests-fuzz.cpp:48-137)
    {
        const std::string s1 = "new york mets", s3 = "the wonderful new york mets";
        const std::string s4 = "new york mets vs atlanta braves", s5 = "atlanta braves vs new york mets";
        const std::string s7 = "new york city mets - atlanta braves";
        CHECK(rapidfuzz::fuzz::token_set_ratio(s4, s5) == 100.0);
        CHECK(rapidfuzz::fuzz::token_set_ratio(std::string("a{"), std::string("{b")) == 50.0);
        CHECK(rapidfuzz::fuzz::partial_token_set_ratio(s4, s7) == 100.0);
        CHECK(rapidfuzz::fuzz::WRatio(s1, s1) == 100.0);
        CHECK(std::fabs(rapidfuzz::fuzz::WRatio(s1, s3) - 90) < 1e-6);
        CHECK(std::fabs(rapidfuzz::fuzz::WRatio(s4, s5) - 95) < 1e-6);
        CHECK(rapidfuzz::fuzz::token_ratio(std::string(""), std::string("")) == 100.0);
        CHECK(rapidfuzz::fuzz::partial_token_ratio(std::string(""), std::string("")) == 100.0);
        CHECK(rapidfuzz::fuzz::WRatio(std::string(""), std::string("")) == 0.0);
        rapidfuzz::fuzz::CachedWRatio<char> cw(s1);
        CHECK(std::fabs(cw.similarity(s3) - 90) < 1e-6);
        rapidfuzz::fuzz::CachedTokenSetRatio<char> cts3(s4);
        CHECK(cts3.similarity(s5) == 100.0);
        rapidfuzz::fuzz::CachedPartialTokenSetRatio<char> cpts3(s4);
        CHECK(cpts3.similarity(s7) == 100.0);
        rapidfuzz::fuzz::CachedTokenRatio<char> ctr(s4);
        CHECK(ctr.similarity(s5) == 100.0);
        rapidfuzz::fuzz::CachedPartialTokenRatio<char> cptr(s4);
        CHECK(cptr.similarity(s7) == 100.0);
    }
    // Multi* (Levenshtein.hpp:297-419) and its errors
    rapidfuzz::experimental::MultiLevenshtein<16> ml(3);
    ml.insert(std::string("kitten"));
    ml.insert(std::string("sitting"));
    ml.insert(std::string(""));
    std::vector<size_t> res(ml.result_count());
    CHECK(res.size() == 16);
    ml.distance(res.data(), res.size(), std::string("sitting"));
    CHECK(res[0] == 3 && res[1] == 0 && res[2] == 7);
    bool threw = false;
    try {
        ml.insert(std::string("x"));
    }
    catch (const std::invalid_argument&) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        std::vector<size_t> small(2);
        ml.distance(small.data(), small.size(), std::string("a"));
    }
    catch (const std::invalid_argument&) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        rapidfuzz::experimental::MultiLevenshtein<8> bad(1, {2, 1, 1});
    }
    catch (const std::invalid_argument&) {
        threw = true;
    }
    CHECK(threw);

    // seeded sweep of every free function and Cached* form against the oracle
    std::mt19937 rng(7);
    const char* alpha = "abcde";
    for (int it = 0; it < 300; ++it) {
        std::string s1, s2;
        int l1 = (int)(rng() % 90), l2 = (int)(rng() % 90);
        for (int i = 0; i < l1; ++i) s1 += alpha[rng() % 5];
        for (int i = 0; i < l2; ++i) s2 += alpha[rng() % 5];
        size_t c = (size_t)(rng() % 40);
        double cf = (rng() % 11) / 10.0;
        LevenshteinWeightTable w{1 + rng() % 2, 1 + rng() % 2, 1 + rng() % 3};
        rfo_params p{(int64_t)w.insert_cost, (int64_t)w.delete_cost, (int64_t)w.replace_cost, 0.1};
        CHECK((int64_t)rapidfuzz::levenshtein_distance(s1, s2, w, c) == oi(RFO_LEVENSHTEIN, RFO_DISTANCE, 0, s1, s2, c, p));
        CHECK(same(rapidfuzz::levenshtein_normalized_similarity(s1, s2, w, cf),
                   of(RFO_LEVENSHTEIN, RFO_NORM_SIMILARITY, 0, s1, s2, cf, p)));
        CHECK((int64_t)rapidfuzz::indel_similarity(s1, s2, c) == oi(RFO_INDEL, RFO_SIMILARITY, 0, s1, s2, c));
        CHECK((int64_t)rapidfuzz::lcs_seq_distance(s1, s2, c) == oi(RFO_LCSSEQ, RFO_DISTANCE, 0, s1, s2, c));
        CHECK((int64_t)rapidfuzz::osa_distance(s1, s2, c) == oi(RFO_OSA, RFO_DISTANCE, 0, s1, s2, c));
        CHECK(same(rapidfuzz::jaro_similarity(s1, s2, cf), of(RFO_JARO, RFO_SIMILARITY, 0, s1, s2, cf)));
        CHECK(same(rapidfuzz::jaro_winkler_distance(s1, s2, 0.1, cf), of(RFO_JARO_WINKLER, RFO_DISTANCE, 0, s1, s2, cf)));
        CHECK(same(rapidfuzz::fuzz::ratio(s1, s2, cf * 100), of(RFO_RATIO, RFO_SIMILARITY, 0, s1, s2, cf * 100)));
        CHECK(same(rapidfuzz::fuzz::partial_ratio(s1, s2, cf * 100),
                   of(RFO_PARTIAL_RATIO, RFO_SIMILARITY, 0, s1, s2, cf * 100)));
        std::string t1, t2; /* whitespace-rich strings for the token scorers */
        for (int i = 0; i < l1; ++i) t1 += " ab\tcd"[rng() % 6];
        for (int i = 0; i < l2; ++i) t2 += " ab\tcd"[rng() % 6];
        CHECK(same(rapidfuzz::fuzz::token_sort_ratio(t1, t2, cf * 100),
                   of(RFO_TOKEN_SORT_RATIO, RFO_SIMILARITY, 0, t1, t2, cf * 100)));
        CHECK(same(rapidfuzz::fuzz::partial_token_sort_ratio(t1, t2, cf * 100),
                   of(RFO_PARTIAL_TOKEN_SORT_RATIO, RFO_SIMILARITY, 0, t1, t2, cf * 100)));
        CHECK(same(rapidfuzz::fuzz::QRatio(t1, t2, cf * 100), of(RFO_QRATIO, RFO_SIMILARITY, 0, t1, t2, cf * 100)));
        CHECK(same(rapidfuzz::fuzz::token_set_ratio(t1, t2, cf * 100),
                   of(RFO_TOKEN_SET_RATIO, RFO_SIMILARITY, 0, t1, t2, cf * 100)));
        CHECK(same(rapidfuzz::fuzz::WRatio(t1, t2, cf * 100), of(RFO_WRATIO, RFO_SIMILARITY, 0, t1, t2, cf * 100)));
        rapidfuzz::fuzz::CachedTokenSortRatio<char> cts2(t1);
        CHECK(same(cts2.similarity(t2, cf * 100), of(RFO_TOKEN_SORT_RATIO, RFO_SIMILARITY, 1, t1, t2, cf * 100)));
        rapidfuzz::CachedOSA<char> co(s1);
        CHECK(same(co.normalized_similarity(s2, cf), of(RFO_OSA, RFO_NORM_SIMILARITY, 1, s1, s2, cf)));
    }
    std::printf("%s (%d failures)\n", failures ? "FAILED" : "ok", failures);
    return failures ? 1 : 0;
}
