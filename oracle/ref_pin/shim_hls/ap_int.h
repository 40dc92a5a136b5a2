// Stand-in for the Xilinx HLS arbitrary-precision integer header, enough for
// the reference's CPU build of its FFT and kernels (test infrastructure; see
// oracle/ref_pin/build_ref.py).  ap_uint<W>: an unsigned W-bit value
// (W <= 64) that wraps mod 2^W, with get_bit / set_bit / range(hi, lo).
#ifndef REF_PIN_AP_INT_H
#define REF_PIN_AP_INT_H
#include <stdint.h>

#include <type_traits>

template <int W>
struct ap_uint {
    static_assert(W > 0 && W <= 64, "stand-in supports W <= 64");
    static constexpr uint64_t kMask = (W == 64) ? ~0ull : ((1ull << W) - 1);
    uint64_t v;

    ap_uint() : v(0) {}
    template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
    ap_uint(T x) : v((uint64_t)(int64_t)x & kMask) {}
    template <int W2>
    ap_uint(const ap_uint<W2>& o) : v(o.v & kMask) {}

    operator uint64_t() const { return v; }

    template <typename T, typename = typename std::enable_if<std::is_arithmetic<T>::value>::type>
    ap_uint& operator=(T x) {
        v = (uint64_t)(int64_t)x & kMask;
        return *this;
    }
    ap_uint& operator++() {
        v = (v + 1) & kMask;
        return *this;
    }
    ap_uint operator++(int) {
        ap_uint t = *this;
        ++*this;
        return t;
    }
    bool get_bit(int i) const { return (v >> i) & 1u; }
    void set_bit(int i, bool b) {
        if (b)
            v |= (1ull << i);
        else
            v &= ~(1ull << i);
        v &= kMask;
    }

    struct range_ref {
        ap_uint* p;
        int hi, lo;
        uint64_t mask() const {
            const int w = hi - lo + 1;
            return (w >= 64) ? ~0ull : ((1ull << w) - 1);
        }
        operator uint64_t() const { return (p->v >> lo) & mask(); }
        range_ref& operator=(uint64_t x) {
            const uint64_t m = mask() << lo;
            p->v = ((p->v & ~m) | ((x << lo) & m)) & kMask;
            return *this;
        }
        range_ref& operator=(const range_ref& o) { return *this = (uint64_t)o; }
    };
    range_ref range(int hi, int lo) { return range_ref{this, hi, lo}; }
    uint64_t range(int hi, int lo) const {
        const int w = hi - lo + 1;
        const uint64_t m = (w >= 64) ? ~0ull : ((1ull << w) - 1);
        return (v >> lo) & m;
    }
};

template <int W>
struct ap_int : ap_uint<W> {
    using ap_uint<W>::ap_uint;
};

#endif
