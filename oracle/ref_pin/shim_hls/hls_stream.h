// Stand-in for the Xilinx HLS stream header (test infrastructure): an
// unbounded FIFO with the << / >> / read / write / empty interface.
#ifndef REF_PIN_HLS_STREAM_H
#define REF_PIN_HLS_STREAM_H
#include <deque>

namespace hls {
template <typename T, int DEPTH = 0>
class stream {
  public:
    void write(const T& x) { q_.push_back(x); }
    T read() {
        T x = q_.front();
        q_.pop_front();
        return x;
    }
    bool empty() const { return q_.empty(); }
    stream& operator<<(const T& x) {
        write(x);
        return *this;
    }
    stream& operator>>(T& x) {
        x = read();
        return *this;
    }

  private:
    std::deque<T> q_;
};
}  // namespace hls
#endif
