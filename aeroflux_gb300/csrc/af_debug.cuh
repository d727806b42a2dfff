// af_debug.cuh -- bounds-checked device pointers for the debug build.
//
// Built with -DAEROFLUX_DEBUG_BOUNDS=1 (the separate debug library), every
// kernel field pointer is a DPtr: the pointer, the base and element count of
// the buffer it points into, and the kernel and slot it serves.  Every load
// and store through it (row pointers and offsets included) checks that the
// element lies inside its buffer; a violation records the first (kernel,
// slot, offset) of this translation unit and a count, and the access goes to
// a sink instead -- no trap, so the context stays usable and the host raises.
// In the product build DPtr<T> is T* and view() returns its argument: the
// kernels compile to the same code as without the wrapper.
#pragma once

#include <stdint.h>

#ifndef AEROFLUX_DEBUG_BOUNDS
#define AEROFLUX_DEBUG_BOUNDS 0
#endif

namespace af {

// Kernel ids of the violation record (one id space for both kernel units).
enum DebugKernel : unsigned {
    DK_BC = 1, DK_DIV, DK_PBC, DK_GRAD, DK_SHADOW, DK_SWEEP_ROWS, DK_SWEEP_TMA, DK_RESIDUAL, DK_CORRECT,
    DK_SMOOTH, DK_RESTRICT, DK_PROLONG, DK_PAIR, DK_VTAIL, DK_SEED, DK_CHECK,
    DK_F64_BC = 32, DK_F64_SWEEP, DK_F64_MACCORMACK, DK_F64_DIV, DK_F64_RBGS, DK_F64_PBC, DK_F64_GRAD, DK_F64_B,
    DK_F64_MAXDIV, DK_F64_MAXABS, DK_F64_KE
};

#if AEROFLUX_DEBUG_BOUNDS

namespace {
__device__ unsigned long long g_dbg_first = ~0ull;  // (kernel << 56) | (slot << 40) | (offset & 2^40-1)
__device__ unsigned int g_dbg_count = 0;
__device__ unsigned long long g_dbg_sink[2];
}  // namespace

__device__ __noinline__ inline void dbg_violation(unsigned kid, int slot, long long off) {
    const unsigned long long key = ((unsigned long long)(kid & 0xFFu) << 56) |
                                   ((unsigned long long)(slot & 0xFFFF) << 40) |
                                   ((unsigned long long)off & 0xFFFFFFFFFFull);
    atomicCAS(&g_dbg_first, ~0ull, key);
    atomicAdd(&g_dbg_count, 1u);
}

template <class T>
struct DPtr {
    T* p;
    T* base;
    long long n;
    unsigned kid;
    int slot;
    __device__ __forceinline__ T& operator[](long long i) const {
        T* q = p + i;
        if (q < base || q >= base + n) {
            dbg_violation(kid, slot, (long long)(q - base));
            return *reinterpret_cast<T*>(g_dbg_sink);
        }
        return *q;
    }
    __device__ __forceinline__ T& operator*() const { return (*this)[0]; }
    __device__ __forceinline__ DPtr operator+(long long o) const { return DPtr{p + o, base, n, kid, slot}; }
    __device__ __forceinline__ DPtr operator-(long long o) const { return DPtr{p - o, base, n, kid, slot}; }
    __device__ __forceinline__ DPtr& operator+=(long long o) {
        p += o;
        return *this;
    }
    __device__ __forceinline__ operator DPtr<const T>() const { return DPtr<const T>{p, base, n, kid, slot}; }
    // Vector access of k consecutive elements starting at element i.
    template <class V>
    __device__ __forceinline__ V& vec(long long i, int k) const {
        T* q = p + i;
        if (q < base || q + k > base + n) {
            dbg_violation(kid, slot, (long long)(q - base));
            return *reinterpret_cast<V*>(g_dbg_sink);
        }
        return *reinterpret_cast<V*>(q);
    }
};

template <class T>
__host__ __device__ __forceinline__ DPtr<T> view(T* p, long long n, unsigned kid, int slot) {
    return DPtr<T>{p, p, n, kid, slot};
}

#define AF_PTR(T) ::af::DPtr<T>
#define AF_RESTRICT
#define AF_VEC(V, ptr, i, k) (ptr).template vec<V>((i), (k))

#else

template <class T>
__host__ __device__ __forceinline__ T* view(T* p, long long, unsigned, int) {
    return p;
}

#define AF_PTR(T) T*
#define AF_RESTRICT __restrict__
#define AF_VEC(V, ptr, i, k) (*reinterpret_cast<V*>((ptr) + (i)))

#endif

}  // namespace af
