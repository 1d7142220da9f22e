/* rfg_token.h -- host front end of the token scorers (token_sort_ratio,
 * partial_token_sort_ratio): sorted_split(s).join() of one string or of a packed set. */
#pragma once
#include <stdint.h>

#include <vector>

namespace rfg {

/* sorted_split(s).join() (common_impl.hpp:162-180, SplittedSentenceView.hpp:71-85): the
 * string is split on whitespace (common_impl.hpp:85-152: one-byte code units know the
 * ASCII set, wider ones the Unicode WS / B / S / Zs set), empty tokens are dropped, the
 * tokens are sorted lexicographically by code unit (compared unsigned) and joined with
 * U+0020.  The result keeps the code-unit width.  Returns the joined length in units;
 * *out holds len * width bytes (plus padding). */
int64_t token_sort_join(const void* s, int64_t len, int width, std::vector<unsigned char>* out);

/* the same for every string of a packed set (offsets validated by the caller); the
 * output offsets start at 0.  Large sets are split over the host threads. */
void token_sort_join_set(const void* data, const int64_t* off, int64_t n, int width,
                         std::vector<unsigned char>* out_data, std::vector<int64_t>* out_off);

/* the token_set_ratio family: per string the concatenation of the parts asked for -- the
 * string itself, its sorted-split join S, the join J of its deduplicated tokens
 * (SplittedSentenceView::dedupe, SplittedSentenceView.hpp:48-54) -- and the three part
 * lengths (0 for a part not asked for), three int32 per string */
void token_parts_set(const void* data, const int64_t* off, int64_t n, int width, bool orig, bool sorted, bool dedup,
                     std::vector<unsigned char>* out_data, std::vector<int64_t>* out_off, std::vector<int32_t>* parts);

} // namespace rfg
