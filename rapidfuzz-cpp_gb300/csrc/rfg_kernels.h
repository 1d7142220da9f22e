/* rfg_kernels.h -- host-side lookup of the kernel instantiations (one translation
 * unit per core family, compiled in parallel). */
#pragma once
#include <stdint.h>

namespace rfg {
/* k_tiles<FAM, CT, W, TOPK>: width in {1,2,4,8}, W in {1,2,4,8}; nullptr when absent */
const void* tiles_kernel_lev(int width, int W, bool topk);
const void* tiles_kernel_lcs(int width, int W, bool topk);
const void* tiles_kernel_osa(int width, int W, bool topk);
const void* tiles_kernel_jaro(int width, int W, bool topk);
/* k_tiles_mq<FAM, CT, NORM, Q, HALF> (unit-weight distances or their normalized chains,
 * several queries per thread; HALF: 32-bit recurrence words for patterns of <= 32 units) */
const void* tiles_mq_kernel_lev(int width, bool norm, bool half);
const void* tiles_mq_kernel_lcs(int width, bool norm, bool half);
const void* tiles_mq_kernel_osa(int width, bool norm, bool half);
/* k_fast<FAM, CT, Q, HALF> (unit-weight distances of one-word patterns, warp tiles over
 * the length-filter range of each window; HALF: 32-bit words for patterns of <= 32 units) */
const void* fast_kernel_lev(int width, bool half);
/* k_fast_hist: the choices' count histograms of the warp tiles' filter */
const void* fast_hist_kernel();
const void* fast_kernel_lcs(int width, bool half);
const void* fast_kernel_osa(int width, bool half);
/* k_band<CT, B, LCS> (banded unit-weight Levenshtein, or with lcs the banded LCS
 * families; B 32-bit words of band in {1, 2, 3, 4, 6, 8, 12, 16}); one-byte choices only,
 * nullptr otherwise */
const void* band_kernel(int width, int B, bool lcs);
const void* band_lcs_kernel(int B);
/* queries per lane of k_fast */
#ifndef RFG_FAST_LCS_Q
#define RFG_FAST_LCS_Q 2 /* queries a lane scores for Indel (2 since the count filter makes the recurrence rare) */
#endif
inline int fast_queries(int fam) { return fam == FAM_LCS ? RFG_FAST_LCS_Q : 2; }
/* k_tiles_mq_jaro<CT, Q> (Jaro / Jaro-Winkler, several queries per thread) */
const void* tiles_mq_kernel_jaro(int width);
/* queries per thread of the several-queries kernels of a family (measured on GB300:
 * two keep Levenshtein / OSA / Jaro state in registers with room for latency hiding,
 * the two-register LCS state takes four) */
inline int mq_queries(int fam) { return fam == FAM_LCS ? 4 : 2; }
/* ... and of the 32-bit-word kernels (measured: twice the queries per thread was slower
 * for Indel and OSA and level for Levenshtein, so the same counts) */
inline int mq_queries_half(int fam) { return mq_queries(fam); }
/* k_generic<FAM, CT, TOPK> */
const void* generic_kernel(int fam, int width, bool topk);
/* k_generic<FAM_TOKEN, CT, TOPK> (its own translation unit) */
const void* token_kernel(int width, bool topk);
/* k_topk_merge */
const void* topk_merge_kernel();
/* k_jaro_tables (per-query JaroTab pre-pass) */
const void* jaro_tables_kernel();
/* k_editops (editops of many pairs, one thread per pair) */
const void* editops_kernel();
/* k_editops_hb (long Levenshtein pairs: the reference's Hirschberg recursion) */
const void* editops_hb_kernel();
/* k_editops_pack (the pairs' operations, packed) */
const void* editops_pack_kernel();
/* k_zero_pairs (QRatio's empty-string rule on a device result matrix) */
const void* zero_pairs_kernel();
} // namespace rfg
