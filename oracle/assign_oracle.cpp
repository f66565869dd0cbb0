// assign_oracle.cpp -- CPU restatement of the equal-size group assignment ISAC
// runs on the multi-reference alignment's peak matrix.
//
// TEST INFRASTRUCTURE ONLY: the checker of gpuisac_assign_groups_device and the
// timed CPU baseline of bench.py's assignment block; nothing in the product
// path links or calls it.
//
// The reference calls Util::assign_groups of EMAN2/SPHIRE (util_sparx.cpp;
// the library is not vendored in the reference and its install script pins no
// version) at bin/sp_isac2_gpu.py:1119 on d[ref * nima + particle] and reads
// the result at bin/sp_isac2_gpu.py:1121-1136.  The algorithm (described by the
// caller's comment at bin/sp_isac2_gpu.py:1114-1118, and by EMAN2's source):
//   * every (reference, particle) pair is ranked by its peak, highest first;
//   * pairs are taken in that order; a pair whose particle is already placed
//     or whose group is closed is skipped, otherwise the particle joins the
//     group;
//   * a group closes when it holds maxasi = nima / nref particles, except the
//     last open group, which closes at maxasi + nima % nref;
//   * the result lists each group's first maxasi members in joining order,
//     group after group, then the extra members of the group that closed last,
//     then that group's index: nima + 1 integers.
// Equal peaks: EMAN2 sorts with std::sort, which leaves the order of equal
// elements unspecified; here (and on the GPU) the pair with the smaller index
// ref * nima + particle comes first.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

extern "C" int orc_assign_groups(const float *d, unsigned nref, unsigned nima, int *id_list_long)
{
    if (!d || !id_list_long || nref == 0 || nima < nref)
        return -1;
    const uint64_t n = (uint64_t)nref * nima;
    if (n > 0xFFFFFFFFull)
        return -1;
    for (uint64_t i = 0; i < n; i++)
        if (std::isnan(d[i]))
            return -2;

    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [d](uint32_t a, uint32_t b) {
        if (d[a] != d[b])
            return d[a] > d[b];
        return a < b;
    });

    const unsigned maxasi = nima / nref, extra = nima % nref;
    std::vector<std::vector<int>> members(nref);
    std::vector<char> closed(nref, 0), placed(nima, 0);
    unsigned open = nref, last = 0;
    uint64_t b = 0;
    while (open > 0) {
        unsigned g = 0, p = 0;
        for (;; b++) {
            if (b >= n)
                return -3;
            g = order[b] / nima;
            p = order[b] % nima;
            if (!placed[p] && !closed[g])
                break;
        }
        members[g].push_back((int)p);
        placed[p] = 1;
        const unsigned cap = open > 1 ? maxasi : maxasi + extra;
        if (members[g].size() >= cap) {
            closed[g] = 1;
            open--;
            last = g;
        }
    }

    size_t o = 0;
    for (unsigned g = 0; g < nref; g++)
        for (unsigned j = 0; j < maxasi; j++)
            id_list_long[o++] = members[g][j];
    for (unsigned j = maxasi; j < maxasi + extra; j++)
        id_list_long[o++] = members[last][j];
    id_list_long[o] = (int)last;
    return 0;
}
