// Persistent schedule of a plan: items -> parts -> warp workers.
//
// The items of one tile are consecutive in the layout.  Runs of them are cut
// into parts of at most part_bytes; a tile larger than that becomes several
// parts, whose partial row sums are combined by the last-arriving worker.
// Parts are assigned to workers by greedy LPT on their bytes (largest part to
// the least loaded worker), so each worker gets a list of whole parts and the
// makespan stays within one part of the mean load.
#include <algorithm>
#include <cstring>
#include <vector>

#include "plan_internal.h"
#include "sable_internal.h"

namespace sable {

struct Part {
    int32_t first, count;  // items [first, first + count) of the layout
    int64_t bytes;
    int64_t tile;
    int32_t index;         // part index within its tile
};

int build_warp_schedule(const Layout &L, int n_workers, int64_t part_bytes, std::vector<WorkRef> &work,
                        std::vector<int> &begin, int64_t &ppartial_floats, int64_t &n_multi, int64_t &n_parts) {
    std::vector<Part> parts;
    const int32_t n = (int32_t)L.items.size();
    for (int32_t i = 0; i < n;) {
        const int64_t tile = L.item_tile[i];
        int32_t j = i;
        int32_t index = 0;
        while (j < n && L.item_tile[j] == tile) {
            Part pt{j, 0, 0, tile, index++};
            while (j < n && L.item_tile[j] == tile && (pt.count == 0 || pt.bytes + L.items[j].bytes <= part_bytes)) {
                pt.bytes += L.items[j].bytes;
                ++pt.count;
                ++j;
            }
            parts.push_back(pt);
        }
        i = j;
    }
    n_parts = (int64_t)parts.size();
    // per tile: number of parts, split counter and partial base
    std::vector<int32_t> tile_nparts, tile_split;
    std::vector<int64_t> tile_base;
    int64_t max_tile = 0;
    for (const Part &pt : parts) max_tile = std::max(max_tile, pt.tile);
    tile_nparts.assign(max_tile + 1, 0);
    tile_split.assign(max_tile + 1, -1);
    tile_base.assign(max_tile + 1, 0);
    for (const Part &pt : parts) tile_nparts[pt.tile]++;
    ppartial_floats = 0;
    n_multi = 0;
    for (const Part &pt : parts) {
        if (tile_nparts[pt.tile] > 1 && pt.index == 0) {
            ItemHeader hd;
            memcpy(&hd, L.records.data() + L.items[pt.first].off, sizeof hd);
            tile_split[pt.tile] = (int32_t)n_multi++;
            tile_base[pt.tile] = ppartial_floats;
            ppartial_floats += (int64_t)tile_nparts[pt.tile] * hd.h;
        }
    }
    // LPT over workers
    const int nw = std::max(1, n_workers);
    std::vector<int32_t> order(parts.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = (int32_t)k;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return parts[a].bytes > parts[b].bytes; });
    std::vector<std::pair<int64_t, int>> heap;
    for (int w = 0; w < nw; ++w) heap.push_back({0, w});
    auto cmp = [](const std::pair<int64_t, int> &a, const std::pair<int64_t, int> &b) {
        return a.first > b.first || (a.first == b.first && a.second > b.second);
    };
    std::make_heap(heap.begin(), heap.end(), cmp);
    std::vector<std::vector<int32_t>> lists(nw);
    for (int32_t k : order) {
        std::pop_heap(heap.begin(), heap.end(), cmp);
        lists[heap.back().second].push_back(k);
        heap.back().first += parts[k].bytes;
        std::push_heap(heap.begin(), heap.end(), cmp);
    }
    work.clear();
    begin.assign(nw + 1, 0);
    for (int w = 0; w < nw; ++w) {
        begin[w] = (int)work.size();
        for (int32_t k : lists[w]) {
            const Part &pt = parts[k];
            for (int32_t c = 0; c < pt.count; ++c) {
                const ItemRef &ir = L.items[pt.first + c];
                WorkRef r;
                memset(&r, 0, sizeof r);
                r.off = ir.off;
                r.bytes = ir.bytes;
                r.flags = (c == 0 ? SABLE_PART_FIRST : 0) | (c == pt.count - 1 ? SABLE_PART_LAST : 0);
                r.part = pt.index;
                r.nparts = tile_nparts[pt.tile];
                r.split = tile_split[pt.tile];
                r.part_base = tile_base[pt.tile];
                work.push_back(r);
            }
        }
    }
    begin[nw] = (int)work.size();
    return SABLE_OK;
}

}  // namespace sable
