// Host stand-in for <cub/cub.cuh> (oracle only).  The reference sorts with
// cub::DeviceRadixSort::SortPairs over all 32 key bits (grid.cuh:91-103), a
// stable LSD sort; this stand-in is the same stable order (std::stable_sort of
// slot indices by key).
#pragma once
#include <algorithm>
#include <vector>
#include <stdint.h>

namespace cub {
struct DeviceRadixSort {
    template <typename K, typename V>
    static int SortPairs(void *temp, size_t &temp_bytes, const K *keys_in, K *keys_out,
                         const V *values_in, V *values_out, int n) {
        if (temp == nullptr) { temp_bytes = 1; return 0; }
        std::vector<int> order(n);
        for (int i = 0; i < n; i++) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return keys_in[a] < keys_in[b]; });
        for (int i = 0; i < n; i++) { keys_out[i] = keys_in[order[i]]; values_out[i] = values_in[order[i]]; }
        return 0;
    }
};
}  // namespace cub
