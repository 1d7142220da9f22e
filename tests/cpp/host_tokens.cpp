/* C entry points over the library's host-side token front end (rfg_token.cpp), for the
 * CPU tests: the sorted-split joins and the [string][S][J] part concatenations that the
 * token scorers upload, compared there with the oracle's restatement. */
#include <string.h>

#include <vector>

#include "rfg_token.h"

extern "C" {

/* token_parts_set; returns the bytes of the concatenations (copied when they fit cap) */
int64_t ht_parts(const void* data, const int64_t* off, int64_t n, int width, int orig, int sorted, int dedup,
                 unsigned char* out, int64_t cap, int64_t* out_off, int32_t* parts)
{
    std::vector<unsigned char> od;
    std::vector<int64_t> oo;
    std::vector<int32_t> pr;
    rfg::token_parts_set(data, off, n, width, orig != 0, sorted != 0, dedup != 0, &od, &oo, &pr);
    memcpy(out_off, oo.data(), (size_t)(n + 1) * 8);
    if (n) memcpy(parts, pr.data(), (size_t)(3 * n) * 4);
    const int64_t bytes = oo[n] * width;
    if (bytes <= cap && bytes) memcpy(out, od.data(), (size_t)bytes);
    return bytes;
}

/* token_sort_join_set */
int64_t ht_join_set(const void* data, const int64_t* off, int64_t n, int width, unsigned char* out, int64_t cap,
                    int64_t* out_off)
{
    std::vector<unsigned char> od;
    std::vector<int64_t> oo;
    rfg::token_sort_join_set(data, off, n, width, &od, &oo);
    memcpy(out_off, oo.data(), (size_t)(n + 1) * 8);
    const int64_t bytes = oo[n] * width;
    if (bytes <= cap && bytes) memcpy(out, od.data(), (size_t)bytes);
    return bytes;
}

/* token_sort_join of one string; returns its length in units */
int64_t ht_join_one(const void* s, int64_t len, int width, unsigned char* out, int64_t cap)
{
    std::vector<unsigned char> od;
    const int64_t n = rfg::token_sort_join(s, len, width, &od);
    if (n * width <= cap && n) memcpy(out, od.data(), (size_t)(n * width));
    return n;
}

} /* extern "C" */
