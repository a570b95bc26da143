// serve_sched.h -- host-side scheduler of the serving loop: device-memory
// pools with first-fit sub-allocation, request slots, FIFO admission and the
// per-tick chunk plan. No CUDA here: the serving runtime (serve.cu) drives
// it against real device pools, and sbg_serve_simulate runs it dry so the
// admission policy can be checked without a GPU.
//
// Continuous batching: every tick, each resident request advances by
// min(its chunk, remaining) fixed RK-Merson steps in the same launch as every
// other resident request; a request whose last step falls in a tick retires
// after it and its memory and slot go back to the pools, where the next
// queued request (strict arrival order, no overtaking) can take them. A
// request's chunk is the scheduler's default, or its own (the serving
// runtime sizes it so that every request's chunk takes about the same time
// on the GPU, so no request waits on a slower neighbour).
#pragma once
#include <cstdint>
#include <deque>
#include <functional>
#include <iterator>
#include <map>
#include <vector>

namespace sbg {

// First-fit allocator over [0, capacity) units, allocations rounded up to a
// multiple of `align` units, coalescing on free.
class FreeList {
public:
    void reset(int64_t capacity, int64_t align) {
        align_ = align;
        cap_ = capacity / align * align;
        free_.clear();
        if (cap_ > 0) free_[0] = cap_;
        used_ = 0;
    }
    int64_t capacity() const { return cap_; }
    int64_t used() const { return used_; }
    int64_t roundUp(int64_t units) const { return (units + align_ - 1) / align_ * align_; }
    // -1 when no free range is large enough.
    int64_t alloc(int64_t units) {
        if (units <= 0) return 0;  // empty allocations share offset 0 and are never freed
        const int64_t need = roundUp(units);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < need) continue;
            const int64_t off = it->first, rest = it->second - need;
            free_.erase(it);
            if (rest > 0) free_[off + need] = rest;
            used_ += need;
            return off;
        }
        return -1;
    }
    void release(int64_t off, int64_t units) {
        if (units <= 0) return;
        int64_t need = roundUp(units);
        used_ -= need;
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + need == next->first) {  // merge with the following range
            need += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {  // merge with the preceding range
                prev->second += need;
                return;
            }
        }
        free_[off] = need;
    }

private:
    std::map<int64_t, int64_t> free_;
    int64_t cap_ = 0, align_ = 256, used_ = 0;
};

// Device footprint of one request, per pool, in the pool's units:
//   rows         body-table rows (one per body, plus one for the level table's end)
//   forces       mobility-force elements
//   state        y elements (with their RK stage planes)
//   scratch      per-body scratch elements of the level-parallel driver
//   loopScratch  FP64 scratch elements of the loop-closure driver
enum PoolKind { kPoolRows = 0, kPoolForces, kPoolState, kPoolScratch, kPoolLoopScratch, kNumPools };
struct Footprint {
    int64_t units[kNumPools] = {0, 0, 0, 0, 0};
};

struct SchedRequest {
    int64_t id = 0;
    Footprint fp;
    int32_t horizon = 0;     // steps requested
    int32_t chunk = 0;       // steps per tick (0 = the scheduler's default)
    // set by the scheduler
    int32_t slot = -1;
    int64_t off[kNumPools] = {0, 0, 0, 0, 0};
    int32_t remaining = 0;
    bool started = false;    // its first chunk has been planned
    int64_t admitTick = -1, doneTick = -1;
};

// One entry of a tick's plan.
struct PlannedChunk {
    int32_t req;     // index into the scheduler's request table
    int32_t steps;   // steps in this tick
    bool first;      // the request's first chunk (Integrator::initialize)
    bool last;       // the request retires after this tick
};

class Scheduler {
public:
    void configure(const int64_t capacity[kNumPools], const int64_t align[kNumPools], int32_t maxSlots, int32_t chunk) {
        for (int k = 0; k < kNumPools; ++k) pools_[k].reset(capacity[k], align[k]);
        freeSlots_.clear();
        for (int32_t s = maxSlots - 1; s >= 0; --s) freeSlots_.push_back(s);
        maxSlots_ = maxSlots;
        chunk_ = chunk;
    }
    int32_t maxSlots() const { return maxSlots_; }
    const FreeList& pool(int k) const { return pools_[k]; }

    // True when the request could be admitted into empty pools at all.
    bool fitsEver(const Footprint& fp) const {
        for (int k = 0; k < kNumPools; ++k)
            if (pools_[k].roundUp(fp.units[k]) > pools_[k].capacity()) return false;
        return maxSlots_ > 0;
    }
    // Queue a request; returns its index in the request table.
    int32_t submit(int64_t id, const Footprint& fp, int32_t horizon, int32_t chunk = 0) {
        SchedRequest r;
        r.id = id;
        r.fp = fp;
        r.horizon = horizon;
        r.chunk = chunk;
        r.remaining = horizon;
        reqs_.push_back(r);
        queue_.push_back((int32_t)reqs_.size() - 1);
        return (int32_t)reqs_.size() - 1;
    }
    // Admit queued requests in arrival order while a slot and room in every
    // pool are free (and `stage`, if given, accepts the request's upload).
    // Returns the indices admitted in this call.
    std::vector<int32_t> admit(int64_t tick, const std::function<bool(int32_t)>& stage = nullptr) {
        std::vector<int32_t> out;
        while (!queue_.empty() && !freeSlots_.empty()) {
            SchedRequest& r = reqs_[queue_.front()];
            int64_t off[kNumPools];
            int k = 0;
            for (; k < kNumPools; ++k) {
                off[k] = pools_[k].alloc(r.fp.units[k]);
                if (off[k] < 0) break;
            }
            if (k == kNumPools && stage) {
                for (int j = 0; j < kNumPools; ++j) r.off[j] = off[j];
                r.slot = freeSlots_.back();
                if (!stage(queue_.front())) k = kNumPools + 1;
            }
            if (k != kNumPools) {  // no room: undo and wait (strict FIFO)
                for (int j = 0; j < k && j < kNumPools; ++j) pools_[j].release(off[j], r.fp.units[j]);
                r.slot = -1;
                break;
            }
            for (int j = 0; j < kNumPools; ++j) r.off[j] = off[j];
            r.slot = freeSlots_.back();
            freeSlots_.pop_back();
            r.admitTick = tick;
            out.push_back(queue_.front());
            active_.push_back(queue_.front());
            queue_.pop_front();
        }
        return out;
    }
    // The chunk of every resident request for this tick; requests whose
    // last chunk this is leave the resident list (their memory stays
    // allocated until retire()). `finish`, if given, may refuse a request's
    // last chunk (no room for its result this tick): the request then stops
    // one step short and finishes in a later tick. The step sequence of a
    // request is the same either way, so its result does not change.
    std::vector<PlannedChunk> plan(int64_t tick, const std::function<bool(int32_t)>& finish = nullptr) {
        std::vector<PlannedChunk> p;
        std::vector<int32_t> keep;
        for (int32_t i : active_) {
            SchedRequest& r = reqs_[i];
            const int32_t c = r.chunk > 0 ? r.chunk : chunk_;
            int32_t steps = r.remaining < c ? r.remaining : c;
            bool last = steps == r.remaining;
            if (last && finish && !finish(i)) {
                if (steps <= 1) {  // nothing to run short of the last step: wait a tick
                    keep.push_back(i);
                    continue;
                }
                --steps;
                last = false;
            }
            p.push_back(PlannedChunk{i, steps, !r.started, last});
            r.started = true;
            r.remaining -= steps;
            if (last) r.doneTick = tick;
            else keep.push_back(i);
        }
        active_.swap(keep);
        return p;
    }
    // Give a finished request's memory and slot back.
    void retire(int32_t i) {
        SchedRequest& r = reqs_[i];
        for (int k = 0; k < kNumPools; ++k) pools_[k].release(r.off[k], r.fp.units[k]);
        freeSlots_.push_back(r.slot);
        r.slot = -1;
    }
    SchedRequest& req(int32_t i) { return reqs_[i]; }
    size_t queued() const { return queue_.size(); }
    size_t resident() const { return active_.size(); }
    int32_t slotsInUse() const { return maxSlots_ - (int32_t)freeSlots_.size(); }

private:
    FreeList pools_[kNumPools];
    std::vector<int32_t> freeSlots_;
    std::vector<SchedRequest> reqs_;
    std::deque<int32_t> queue_;
    std::vector<int32_t> active_;
    int32_t maxSlots_ = 0, chunk_ = 64;
};

}  // namespace sbg
