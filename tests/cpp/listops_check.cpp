/* Reads operation lists on stdin and prints the list operations of the C++ drop-in
 * header's Editops / Opcodes (slice, remove_slice, reverse, inverse, remove_subsequence)
 * for the CPU tests, which compare them with the reference's (listops.json).  Input:
 * the case count, then per case: which start stop step n, n x (type src dest), src_len
 * dest_len.  Output per case: "err" where the header throws invalid_argument, else the
 * record count, the records (3 or 5 numbers) and the two lengths. */
#include <cstdio>
#include <stdexcept>

#include <rapidfuzz_gb300/rapidfuzz.hpp>

namespace rf = rapidfuzz_gb300;

static long long next()
{
    long long v = 0;
    if (std::scanf("%lld", &v) != 1) return -1;
    return v;
}

int main()
{
    const long long cases = next();
    for (long long c = 0; c < cases; ++c) {
        const int which = (int)next(), start = (int)next(), stop = (int)next(), step = (int)next();
        const long long n = next();
        rf::Editops e;
        for (long long k = 0; k < n; ++k) {
            const long long t = next(), s = next(), d = next();
            e.emplace_back((rf::EditType)t, (size_t)s, (size_t)d);
        }
        e.set_src_len((size_t)next());
        e.set_dest_len((size_t)next());
        try {
            if (which < 10) {
                rf::Editops r;
                if (which == 0) r = e.slice(start, stop, step);
                else if (which == 1) {
                    r = e;
                    r.remove_slice(start, stop, step);
                }
                else if (which == 2) r = e.reverse();
                else if (which == 3) r = e.inverse();
                else r = e.remove_subsequence(e.slice(start, stop, step));
                std::printf("%zu", r.size());
                for (const auto& x : r) std::printf(" %d %zu %zu", (int)x.type, x.src_pos, x.dest_pos);
                std::printf(" %zu %zu\n", r.get_src_len(), r.get_dest_len());
            }
            else {
                const rf::Opcodes o(e);
                rf::Opcodes r;
                if (which == 10) r = o.slice(start, stop, step);
                else if (which == 12) r = o.reverse();
                else r = o.inverse();
                std::printf("%zu", r.size());
                for (const auto& x : r)
                    std::printf(" %d %zu %zu %zu %zu", (int)x.type, x.src_begin, x.src_end, x.dest_begin, x.dest_end);
                std::printf(" %zu %zu\n", r.get_src_len(), r.get_dest_len());
            }
        }
        catch (const std::invalid_argument&) {
            std::printf("err\n");
        }
    }
    return 0;
}
