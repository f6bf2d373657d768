// Host-side helpers shared by the qmbx translation units.
#pragma once

#include <stdint.h>

#include <cstddef>

#include "format.h"

namespace qmbx {

// Record an error message for qmbx_last_error() and return status.
int fail(int status, const char* fmt, ...);
void clear_error();

// Bump allocator over a caller-provided workspace.  With base == nullptr it
// only measures, which is how the *_workspace queries are answered.
struct Arena {
    char* base;
    uint64_t cap;
    uint64_t used = 0;
    Arena(void* b, uint64_t c) : base(static_cast<char*>(b)), cap(c) {}
    template <class T>
    T* take(uint64_t count) {
        uint64_t bytes = (count * sizeof(T) + QMBX_ALIGN - 1) / QMBX_ALIGN * QMBX_ALIGN;
        if (bytes == 0) bytes = QMBX_ALIGN;
        T* p = base ? reinterpret_cast<T*>(base + used) : nullptr;
        used += bytes;
        return p;
    }
    bool fits() const { return base == nullptr || used <= cap; }
};

inline const qmbx_table_header* header_of(const void* table_host) {
    return static_cast<const qmbx_table_header*>(table_host);
}

}  // namespace qmbx
