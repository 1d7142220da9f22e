/* Reads operation lists on stdin and prints what the C++ drop-in header makes of them:
 * Opcodes(Editops), Opcodes::as_editops() and the two applies.  Header-only classes, no
 * device call: the CPU tests compare the output with the reference's (opcodes.json).
 * Input per case: n, n x (type src dest), la, la units, lb, lb units; first the case count. */
#include <cstdio>
#include <vector>

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
        rf::Editops e;
        const long long n = next();
        for (long long k = 0; k < n; ++k) {
            const long long t = next(), s = next(), d = next();
            e.emplace_back((rf::EditType)t, (size_t)s, (size_t)d);
        }
        std::vector<unsigned char> s1((size_t)next()), s2;
        for (auto& x : s1) x = (unsigned char)next();
        s2.resize((size_t)next());
        for (auto& x : s2) x = (unsigned char)next();
        e.set_src_len(s1.size());
        e.set_dest_len(s2.size());
        const rf::Opcodes o(e);
        std::printf("%zu", o.size());
        for (const auto& x : o)
            std::printf(" %d %zu %zu %zu %zu", (int)x.type, x.src_begin, x.src_end, x.dest_begin, x.dest_end);
        const rf::Editops b = o.as_editops();
        std::printf("\n%zu", b.size());
        for (const auto& x : b) std::printf(" %d %zu %zu", (int)x.type, x.src_pos, x.dest_pos);
        const std::vector<unsigned char> ea = rf::editops_apply_vec<unsigned char>(e, s1, s2);
        const std::vector<unsigned char> oa = rf::opcodes_apply_vec<unsigned char>(o, s1, s2);
        std::printf("\n%zu", ea.size());
        for (unsigned char x : ea) std::printf(" %d", x);
        std::printf("\n%zu", oa.size());
        for (unsigned char x : oa) std::printf(" %d", x);
        std::printf("\n");
    }
    return 0;
}
