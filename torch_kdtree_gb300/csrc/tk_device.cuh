// Device-side building blocks shared by the KNN kernels.
//
//  * PointRec<T>: a reference point as stored in HBM -- three coordinates
//    (zero-padded below three dimensions) and the ORIGINAL index in the
//    fourth slot, so one 16-byte (f32) load yields everything a candidate
//    needs and the remap through shuffled_inds (torch_kdtree/nn_distance.py:109)
//    disappears.
//  * Key<T>: (squared distance, original index) packed so that an unsigned
//    compare orders candidates by distance, then by lower index.
//  * sqdist<T, D>: the reference's distance arithmetic, bit for bit:
//    d_c = q_c - r_c, s = ((0 + d0*d0) + d1*d1) + d2*d2, every operation
//    rounded separately (src/kdtree.hpp:546-591).  The _rn intrinsics keep
//    the compiler from fusing multiply and add.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tk {

template <typename T>
struct alignas(4 * sizeof(T)) PointRec {
    T x, y, z, w;  // w: raw bits of the original index (of a leaf range bound in box records)
};

__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

__device__ __forceinline__ PointRec<float> load_rec(const PointRec<float>* p) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    return PointRec<float>{v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ PointRec<double> load_rec(const PointRec<double>* p) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    return PointRec<double>{a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ uint32_t rec_index(const PointRec<float>& r) { return __float_as_uint(r.w); }
__device__ __forceinline__ uint32_t rec_index(const PointRec<double>& r) {
    return uint32_t(__double_as_longlong(r.w));
}

// 32-byte (256-bit) stores to global memory; p must be 32-byte aligned.  A
// lane that writes its own result row stores it in whole 32-byte sectors:
// rows written into host memory over the CPU link move at ~140 GB/s this
// way against ~40 GB/s as 16-byte pieces (measured on GB300).
__device__ __forceinline__ void st_v8(float* p, float a, float b, float c, float d, float e, float f, float g,
                                      float h) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a), "f"(b), "f"(c),
                 "f"(d), "f"(e), "f"(f), "f"(g), "f"(h)
                 : "memory");
}
__device__ __forceinline__ void st_v8(int32_t* p, int32_t a, int32_t b, int32_t c, int32_t d, int32_t e,
                                      int32_t f, int32_t g, int32_t h) {
    asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(a), "r"(b), "r"(c),
                 "r"(d), "r"(e), "r"(f), "r"(g), "r"(h)
                 : "memory");
}
__device__ __forceinline__ void st_v4(double* p, double a, double b, double c, double d) {
    asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p), "d"(a), "d"(b), "d"(c), "d"(d) : "memory");
}

template <typename T, int D>
__device__ __forceinline__ T sqdist(const T (&q)[D], const PointRec<T>& p) {
    const T d0 = sub_rn(q[0], p.x);
    T acc = mul_rn(d0, d0);
    if (D > 1) {
        const T d1 = sub_rn(q[1], p.y);
        acc = add_rn(acc, mul_rn(d1, d1));
    }
    if (D > 2) {
        const T d2 = sub_rn(q[2], p.z);
        acc = add_rn(acc, mul_rn(d2, d2));
    }
    return acc;
}

// ------------------------------------------------------------------ keys --

template <typename T>
struct Key;

// f32: (distance bits << 32) | index.  Distances are >= +0, so their bit
// patterns order like the values; NaN (0x7fc...) sorts above +inf.
template <>
struct Key<float> {
    unsigned long long v;
    static __device__ __forceinline__ Key make(float d, uint32_t i) {
        return Key{(static_cast<unsigned long long>(__float_as_uint(d)) << 32) | i};
    }
    // worst possible real entry: +inf distance, index 2^32-1
    static __device__ __forceinline__ Key sentinel() { return Key{0x7F800000FFFFFFFFull}; }
    // front padding below every real key (see the top-k list below)
    static __device__ __forceinline__ Key pad() { return Key{0ull}; }
    __device__ __forceinline__ float dist() const { return __uint_as_float(uint32_t(v >> 32)); }
    __device__ __forceinline__ uint32_t index() const { return uint32_t(v); }
    __device__ __forceinline__ bool le(const Key& o) const { return v <= o.v; }
    __device__ __forceinline__ bool lt(const Key& o) const { return v < o.v; }
    __device__ __forceinline__ Key shfl(unsigned mask, int src, int width) const {
        return Key{__shfl_sync(mask, v, src, width)};
    }
    __device__ __forceinline__ Key shfl_up(unsigned mask, int delta, int width) const {
        return Key{__shfl_up_sync(mask, v, delta, width)};
    }
    __device__ __forceinline__ Key select(bool c, const Key& o) const { return c ? *this : o; }
};

// f64: distance bits and index side by side, compared lexicographically.
template <>
struct Key<double> {
    unsigned long long d;
    uint32_t i;
    static __device__ __forceinline__ Key make(double dist, uint32_t idx) {
        return Key{static_cast<unsigned long long>(__double_as_longlong(dist)), idx};
    }
    static __device__ __forceinline__ Key sentinel() { return Key{0x7FF0000000000000ull, 0xFFFFFFFFu}; }
    static __device__ __forceinline__ Key pad() { return Key{0ull, 0u}; }
    __device__ __forceinline__ double dist() const { return __longlong_as_double((long long)d); }
    __device__ __forceinline__ uint32_t index() const { return i; }
    __device__ __forceinline__ bool le(const Key& o) const { return d < o.d || (d == o.d && i <= o.i); }
    __device__ __forceinline__ bool lt(const Key& o) const { return d < o.d || (d == o.d && i < o.i); }
    __device__ __forceinline__ Key shfl(unsigned mask, int src, int width) const {
        return Key{__shfl_sync(mask, d, src, width), __shfl_sync(mask, i, src, width)};
    }
    __device__ __forceinline__ Key shfl_up(unsigned mask, int delta, int width) const {
        return Key{__shfl_up_sync(mask, d, delta, width), __shfl_up_sync(mask, i, delta, width)};
    }
    __device__ __forceinline__ Key select(bool c, const Key& o) const { return c ? *this : o; }
};

// ------------------------------------------------------------ top-k list --
//
// A sorted list of KMAX = G * R keys held in registers by a group of G lanes:
// slot s lives on lane s % G, register s / G.  For a query asking for k <= KMAX
// neighbours the first KMAX - k slots hold pad() (below every real key) and
// the rest start at sentinel(); inserting a candidate c shifts every slot
// above c one place up and drops the last, so the worst kept entry is always
// slot KMAX - 1 (lane G-1, register R-1) and pads never move.  With G == 1 the
// list is an ordinary per-thread register array.
template <typename T, int G, int R>
struct TopK {
    Key<T> slot[R];

    __device__ __forceinline__ void init(int k, int gl) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int s = r * G + gl;
            slot[r] = (s < G * R - k) ? Key<T>::pad() : Key<T>::sentinel();
        }
    }

    // Insert c (the same value on every lane of the group).  gmask: the
    // group's lanes; gl: this lane's rank in the group.
    // Slots are rewritten from the top down, so every step still reads the
    // old values of slot r and r - 1 and no second copy of the list is live.
    __device__ __forceinline__ void insert(const Key<T>& c, unsigned gmask, int gl) {
#pragma unroll
        for (int r = R - 1; r >= 0; --r) {
            const Key<T> old = slot[r];
            Key<T> prev;
            bool has_prev;
            if (G == 1) {
                prev = r > 0 ? slot[r - 1] : Key<T>::pad();
                has_prev = r > 0;
            } else {
                const Key<T> up = old.shfl_up(gmask, 1, G);
                const Key<T> wrap = r > 0 ? slot[r - 1].shfl(gmask, G - 1, G) : Key<T>::pad();
                prev = gl == 0 ? wrap : up;
                has_prev = !(gl == 0 && r == 0);
            }
            const bool keep = old.le(c);
            const bool take = !has_prev || prev.le(c);
            slot[r] = keep ? old : (take ? c : prev);
        }
    }

    // G == 32: merge one candidate per lane (sentinel where none) at once:
    // bitonic sort of the 32 candidates across the warp, element-wise min of
    // the list's last 32 slots with the reversed sorted batch (the list and the
    // batch, padded with sentinels to the list's length, give a bitonic
    // sequence holding the 32 R smallest of both), then a bitonic clean-up.
    // Same result as inserting the candidates one by one.
    __device__ __forceinline__ void merge_warp_batch(Key<T> x, int lane) {
        static_assert(G == 32, "one candidate per lane of a full warp");
#pragma unroll
        for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                const Key<T> p = x.shfl(0xFFFFFFFFu, lane ^ stride, 32);
                const bool take_min = ((lane & size) == 0) == ((lane & stride) == 0);
                const bool p_less = p.lt(x);
                x = (take_min == p_less) ? p : x;
            }
        }
        const Key<T> b = x.shfl(0xFFFFFFFFu, 31 - lane, 32);
        slot[R - 1] = b.lt(slot[R - 1]) ? b : slot[R - 1];
#pragma unroll
        for (int stride = 16 * R; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                const int rs = stride / 32;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if ((r & rs) == 0) {
                        const Key<T> a = slot[r], c = slot[r + rs];
                        const bool sw = c.lt(a);
                        slot[r] = sw ? c : a;
                        slot[r + rs] = sw ? a : c;
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const Key<T> p = slot[r].shfl(0xFFFFFFFFu, lane ^ stride, 32);
                    const bool lower = (lane & stride) == 0;
                    const bool p_less = p.lt(slot[r]);
                    slot[r] = (lower == p_less) ? p : slot[r];
                }
            }
        }
    }

    __device__ __forceinline__ Key<T> worst(unsigned gmask) const {
        if (G == 1) return slot[R - 1];
        return slot[R - 1].shfl(gmask, G - 1, G);
    }

    // Write the k live slots of this lane to row `row` of the outputs.
    __device__ __forceinline__ void store(int k, int gl, T* out_d, int32_t* out_i, long long row) const {
        if constexpr (G == 1 && R % 8 == 0) {
            // all R slots live and both rows 32-byte aligned: whole-sector stores
            T* pd = out_d + row * k;
            int32_t* pi = out_i + row * k;
            if (k == R && ((reinterpret_cast<uintptr_t>(pd) | reinterpret_cast<uintptr_t>(pi)) & 31) == 0) {
#pragma unroll
                for (int r = 0; r < R; r += 8) {
                    if constexpr (sizeof(T) == 4) {
                        st_v8(pd + r, slot[r].dist(), slot[r + 1].dist(), slot[r + 2].dist(), slot[r + 3].dist(),
                              slot[r + 4].dist(), slot[r + 5].dist(), slot[r + 6].dist(), slot[r + 7].dist());
                    } else {
                        st_v4(pd + r, slot[r].dist(), slot[r + 1].dist(), slot[r + 2].dist(), slot[r + 3].dist());
                        st_v4(pd + r + 4, slot[r + 4].dist(), slot[r + 5].dist(), slot[r + 6].dist(),
                              slot[r + 7].dist());
                    }
                    st_v8(pi + r, int32_t(slot[r].index()), int32_t(slot[r + 1].index()),
                          int32_t(slot[r + 2].index()), int32_t(slot[r + 3].index()), int32_t(slot[r + 4].index()),
                          int32_t(slot[r + 5].index()), int32_t(slot[r + 6].index()), int32_t(slot[r + 7].index()));
                }
                return;
            }
        }
        if constexpr (G == 1 && R % 4 == 0) {
            // all R slots live and both rows 16-byte aligned: 16-byte stores
            T* pd = out_d + row * k;
            int32_t* pi = out_i + row * k;
            if (k == R && ((reinterpret_cast<uintptr_t>(pd) | reinterpret_cast<uintptr_t>(pi)) & 15) == 0) {
#pragma unroll
                for (int r = 0; r < R; r += 4) {
                    if constexpr (sizeof(T) == 4) {
                        *reinterpret_cast<float4*>(pd + r) =
                            make_float4(slot[r].dist(), slot[r + 1].dist(), slot[r + 2].dist(), slot[r + 3].dist());
                    } else {
                        *reinterpret_cast<double2*>(pd + r) = make_double2(slot[r].dist(), slot[r + 1].dist());
                        *reinterpret_cast<double2*>(pd + r + 2) = make_double2(slot[r + 2].dist(), slot[r + 3].dist());
                    }
                    *reinterpret_cast<int4*>(pi + r) =
                        make_int4(int32_t(slot[r].index()), int32_t(slot[r + 1].index()), int32_t(slot[r + 2].index()),
                                  int32_t(slot[r + 3].index()));
                }
                return;
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int s = r * G + gl;
            const int o = s - (G * R - k);
            if (o >= 0) {
                out_d[row * k + o] = slot[r].dist();
                out_i[row * k + o] = int32_t(slot[r].index());
            }
        }
    }
};

// Offer the candidates of a group (one per lane; sentinel() when a lane has
// none) to the group's list, in lane order.  Returns the new worst key.
template <typename T, int G, int R>
__device__ __forceinline__ Key<T> offer(TopK<T, G, R>& list, const Key<T>& mine, Key<T> worst,
                                        unsigned gmask, int gl, int gbase) {
    if (G == 1) {
        if (mine.lt(worst)) {
            list.insert(mine, gmask, gl);
            worst = list.worst(gmask);
        }
        return worst;
    }
    unsigned m = __ballot_sync(gmask, mine.lt(worst));
    if constexpr (G < 32) m = (m >> gbase) & ((1u << G) - 1u);
    if constexpr (G == 32) {
        if (__popc(m) >= 8) {  // many at once (while the list fills): one sorted merge
            list.merge_warp_batch(mine.lt(worst) ? mine : Key<T>::sentinel(), gl);
            return list.worst(gmask);
        }
    }
    while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const Key<T> c = mine.shfl(gmask, src, G);
        if (c.lt(worst)) {
            list.insert(c, gmask, gl);
            worst = list.worst(gmask);
        }
    }
    return worst;
}

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
    if constexpr (G == 32) {
        return 0xFFFFFFFFu;
    } else {
        const int gbase = lane & ~(G - 1);
        return ((1u << G) - 1u) << gbase;
    }
}

// Cost class of a query for the launch order (smaller = costlier).  The
// squared distance from the query to the farthest corner of its home leaf's
// bounding box bounds its distance to every point of that leaf, so it tracks
// the radius the search must cover: queries far from their leaf's points
// (outside the cloud, in sparse regions) scan many more leaves.  Its float
// exponent and top mantissa bit give half-octave classes, 2^-63 .. 2^64
// mapped onto 255 .. 0; an empty leaf or a non-finite value gets the last
// class.
__device__ __forceinline__ uint32_t cost_class(float far2) {
    if (!(far2 <= 3.0e38f)) return 255u;
    const uint32_t bucket = __float_as_uint(far2) >> 22;  // exponent and top mantissa bit
    const uint32_t c = bucket < 128u ? 0u : (bucket - 128u > 255u ? 255u : bucket - 128u);
    return 255u - c;
}

}  // namespace tk
