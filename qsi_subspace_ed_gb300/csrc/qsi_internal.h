// Internal helpers shared by the host (.cpp) and device (.cu) translation units.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <string>
#include "../../include/qsi_ed.h"

namespace qsi {

// Sets the calling thread's last-error text and returns the status unchanged.
qsi_status fail(qsi_status st, const char* fmt, ...);

using u128 = unsigned __int128;

inline u128 make_u128(uint64_t lo, uint64_t hi) { return ((u128)hi << 64) | lo; }
inline uint64_t lo64(u128 v) { return (uint64_t)v; }
inline uint64_t hi64(u128 v) { return (uint64_t)(v >> 64); }
inline int popc128(u128 v) { return __builtin_popcountll(lo64(v)) + __builtin_popcountll(hi64(v)); }

// Exceptions never leave an extern "C" function: this wrapper turns them into statuses.
template <class F>
qsi_status guarded(F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(QSI_OOM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(QSI_INVALID_ARG, "%s", e.what());
    } catch (...) {
        return fail(QSI_INVALID_ARG, "unknown exception");
    }
}

}  // namespace qsi
