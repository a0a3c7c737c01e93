// Per-context cache of a device symbol's address (host code only).
//
// A `__device__` array's device address belongs to a CUDA context: the
// primary context of a device, a context a driver-API caller created itself,
// or the new primary context after cudaDeviceReset each have their own.  The
// no-alloc entry point caches the address of its scratch array keyed by the
// current context's unique id (cuCtxGetId, never reused within a process) and
// looks it up again for a context it has not seen.  The logic is kept apart
// from the CUDA calls so that it can be tested on a host without a GPU.
#pragma once

namespace tg {

struct CtxAddrCache {
    static constexpr int kEntries = 64;
    struct Entry {
        unsigned long long id;
        void* ptr;
    } e[kEntries] = {};
    int count = 0, next = 0;
};

// `ctx_id()` returns the current context's id (0: the thread has no current
// context); `lookup(void**)` returns 0 and the address in the current context,
// making a context current if there was none.  A lookup happens whenever the
// current context's id is not cached; an id of 0 is never cached.  A full
// cache drops its oldest entry.  Returns lookup's nonzero status on failure.
template <class IdFn, class LookupFn> int ctx_cached_address(CtxAddrCache& c, IdFn ctx_id, LookupFn lookup, void** out)
{
    unsigned long long id = ctx_id();
    if (id != 0)
        for (int k = 0; k < c.count; ++k)
            if (c.e[k].id == id) {
                *out = c.e[k].ptr;
                return 0;
            }
    void* p = nullptr;
    const int st = lookup(&p);
    if (st != 0) return st;
    if (id == 0) id = ctx_id();
    if (id != 0) {
        c.e[c.next] = CtxAddrCache::Entry{id, p};
        c.next = (c.next + 1) % CtxAddrCache::kEntries;
        if (c.count < CtxAddrCache::kEntries) ++c.count;
    }
    *out = p;
    return 0;
}

} // namespace tg
