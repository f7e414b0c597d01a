// boost::iostreams::filtering_streambuf stand-in for relativity.cc: a
// pass-through stream buffer over the pushed istream (no gzip support; the
// oracle feeds uncompressed text).
#pragma once
#include <istream>
#include <stdexcept>
#include <streambuf>
namespace boost {
namespace iostreams {
struct input {};
struct gzip_decompressor {};
template <class Mode>
class filtering_streambuf : public std::streambuf {
 public:
  void push(const gzip_decompressor&) { throw std::runtime_error("gzip input not supported"); }
  void push(std::istream& is) { src_ = is.rdbuf(); }

 protected:
  int_type underflow() override {
    if (!src_) return traits_type::eof();
    std::streamsize n = src_->sgetn(buf_, sizeof buf_);
    if (n <= 0) return traits_type::eof();
    setg(buf_, buf_, buf_ + n);
    return traits_type::to_int_type(buf_[0]);
  }

 private:
  std::streambuf* src_ = nullptr;
  char buf_[1 << 16];
};
}  // namespace iostreams
}  // namespace boost
