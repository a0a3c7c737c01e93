// Host-only test of tg::ctx_cached_address (noalloc_ctx_cache.h) with a fake
// context source: the lookup runs once per context, again after the context
// changes (a driver-API caller's own context, the new primary context after a
// device reset), never caches a thread with no context, and reports a failed
// lookup.  Prints "ok" and exits 0 on success.
#include <cstdio>

#include "noalloc_ctx_cache.h"

namespace {

unsigned long long g_ctx = 0;  // the fake current context's id (0: none)
int g_lookups = 0;
bool g_fail = false;

// The address a context holds the symbol at: distinct per context.
void* addr_of(unsigned long long ctx) { return reinterpret_cast<void*>(0x1000ull * (ctx + 1)); }

int get(tg::CtxAddrCache& c, void** out)
{
    return tg::ctx_cached_address(
        c, [] { return g_ctx; },
        [](void** p) {
            ++g_lookups;
            if (g_fail) return 1;
            if (g_ctx == 0) g_ctx = 7;  // the lookup makes the primary context current
            *p = addr_of(g_ctx);
            return 0;
        },
        out);
}

int fails = 0;
void check(bool ok, const char* what)
{
    if (!ok) {
        std::printf("FAIL: %s\n", what);
        ++fails;
    }
}

} // namespace

int main()
{
    tg::CtxAddrCache c;
    void* p = nullptr;
    // first call in context 1 looks the address up, the second reuses it
    g_ctx = 1;
    check(get(c, &p) == 0 && p == addr_of(1) && g_lookups == 1, "first lookup in context 1");
    check(get(c, &p) == 0 && p == addr_of(1) && g_lookups == 1, "cached in context 1");
    // a caller's own context: a new lookup, with that context's address
    g_ctx = 2;
    check(get(c, &p) == 0 && p == addr_of(2) && g_lookups == 2, "lookup repeated in context 2");
    // back to context 1: still cached
    g_ctx = 1;
    check(get(c, &p) == 0 && p == addr_of(1) && g_lookups == 2, "context 1 still cached");
    // a device reset gives the primary context a new id: looked up again
    g_ctx = 3;
    check(get(c, &p) == 0 && p == addr_of(3) && g_lookups == 3, "lookup repeated after a reset");
    // no current context: the lookup makes one current and its id is cached afterwards
    g_ctx = 0;
    check(get(c, &p) == 0 && p == addr_of(7) && g_lookups == 4, "lookup on a thread without a context");
    check(get(c, &p) == 0 && p == addr_of(7) && g_lookups == 4, "cached once the context is current");
    // a failed lookup is reported and caches nothing
    g_ctx = 9;
    g_fail = true;
    check(get(c, &p) == 1, "failed lookup reported");
    g_fail = false;
    check(get(c, &p) == 0 && p == addr_of(9) && g_lookups == 6, "lookup after a failure");
    // more contexts than entries: the oldest are dropped, every answer stays right
    for (unsigned long long k = 100; k < 100 + 2 * tg::CtxAddrCache::kEntries; ++k) {
        g_ctx = k;
        check(get(c, &p) == 0 && p == addr_of(k), "many contexts");
    }
    const int before = g_lookups;
    g_ctx = 1;
    check(get(c, &p) == 0 && p == addr_of(1) && g_lookups == before + 1, "evicted context looked up again");
    if (fails) return 1;
    std::printf("ok\n");
    return 0;
}
