// lp_umap.h -- the iteration order of the reference's per-contig label
// tally.  label_propagation (cuda/Cuda2.cu:600-621) sums neighbour scores in
// a std::unordered_map<size_t, double> and takes std::max_element over it, so
// among labels with exactly equal scores the one met first in the map's
// iteration order wins.  This header reproduces that order for the C++
// library this project is built and checked against (GNU libstdc++, as
// observed by running it): identity hash, bucket = key mod bucket count, a
// singly linked node list in which a node joins at the head of its bucket's
// run when the bucket is occupied and at the front of the list when it is
// not, and a rehash -- before the insertion that would exceed the bucket
// count -- that re-inserts the nodes in list order under the same rule.  The
// bucket counts are the sequence the library grows through.  A test checks
// the order against std::unordered_map itself on random key sets.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define LPU_HD __host__ __device__ __forceinline__
#else
#define LPU_HD inline
#endif

namespace lpu {

constexpr int kSizes = 19;
// bucket counts (the table grows to the next one when its size would exceed
// the current one)
LPU_HD uint32_t bucket_count(int i) {
    constexpr uint32_t b[kSizes] = {13,     29,     59,     127,    257,    541,     1109,    2357,    5087,   10273,
                                    20753,  42043,  85229,  172933, 351061, 712697, 1447153, 2938679, 5967347};
    return b[i];
}

// the largest number of keys this header orders
constexpr uint32_t kMaxKeys = 5967347;

// Buckets needed for k keys (the bb scratch of order()).
LPU_HD uint32_t buckets_for(uint32_t k) {
    int i = 0;
    while (i + 1 < kSizes && k > bucket_count(i)) ++i;
    return bucket_count(i);
}

// Iteration order after inserting the distinct keys key[0..k) in turn,
// returned as a linked list over key indices: the head index, then nxt[i]
// (-1 ends).  Scratch: nxt[k],
// bb[buckets_for(k)] (bucket -> index of the node before its first node;
// -2 the list head, -1 empty).  k <= kMaxKeys.
template <class Key>
LPU_HD int32_t order(const Key* key, uint32_t k, int32_t* nxt, int32_t* bb) {
    int32_t head = -1;
    int bi = 0;
    uint32_t B = bucket_count(0);
    for (uint32_t b = 0; b < B; ++b) bb[b] = -1;
    for (uint32_t x = 0; x < k; ++x) {
        if (x + 1 > B) {  // rehash: the list re-inserted in its order
            ++bi;
            B = bucket_count(bi);
            for (uint32_t b = 0; b < B; ++b) bb[b] = -1;
            int32_t p = head;
            head = -1;
            while (p >= 0) {
                const int32_t nx = nxt[p];
                const uint32_t b = (uint32_t)((uint64_t)key[p] % B);
                if (bb[b] == -1) {
                    nxt[p] = head;
                    head = p;
                    bb[b] = -2;
                    if (nxt[p] >= 0) bb[(uint32_t)((uint64_t)key[nxt[p]] % B)] = p;
                } else if (bb[b] == -2) {
                    nxt[p] = head;
                    head = p;
                } else {
                    nxt[p] = nxt[bb[b]];
                    nxt[bb[b]] = p;
                }
                p = nx;
            }
        }
        const uint32_t b = (uint32_t)((uint64_t)key[x] % B);
        if (bb[b] == -1) {
            nxt[x] = head;
            head = (int32_t)x;
            bb[b] = -2;
            if (nxt[x] >= 0) bb[(uint32_t)((uint64_t)key[nxt[x]] % B)] = (int32_t)x;
        } else if (bb[b] == -2) {
            nxt[x] = head;
            head = (int32_t)x;
        } else {
            nxt[x] = nxt[bb[b]];
            nxt[bb[b]] = (int32_t)x;
        }
    }
    return head;
}

}  // namespace lpu
