// Stand-in for boost::iostreams::filtering_istream / filtering_ostream with an
// optional gzip stage, as used by the reference's .cfg(.gz) reader and writer.
// The input side slurps the pushed file (inflating it through zlib when a gzip
// stage was pushed) into a string buffer; the output side buffers everything and
// writes it (deflated when requested) to the pushed file when destroyed.
// Test infrastructure only.
#ifndef LMC_ORACLE_SHIM_BOOST_IOSTREAMS_FILTERING_STREAM_
#define LMC_ORACLE_SHIM_BOOST_IOSTREAMS_FILTERING_STREAM_
#include <fstream>
#include <iterator>
#include <sstream>
#include <stdexcept>
#include <string>
#include <zlib.h>
#include "boost/iostreams/filter/gzip.hpp"
namespace boost { namespace iostreams {
namespace shim {
inline std::string Inflate(const std::string &in) {
  z_stream zs{};
  if (inflateInit2(&zs, 16 + MAX_WBITS) != Z_OK) throw std::runtime_error("zlib inflateInit2 failed");
  zs.next_in = reinterpret_cast<Bytef *>(const_cast<char *>(in.data()));
  zs.avail_in = static_cast<uInt>(in.size());
  std::string out;
  char buf[1 << 16];
  int rc;
  do {
    zs.next_out = reinterpret_cast<Bytef *>(buf);
    zs.avail_out = sizeof(buf);
    rc = inflate(&zs, Z_NO_FLUSH);
    if (rc != Z_OK && rc != Z_STREAM_END) { inflateEnd(&zs); throw std::runtime_error("zlib inflate failed"); }
    out.append(buf, sizeof(buf) - zs.avail_out);
  } while (rc != Z_STREAM_END);
  inflateEnd(&zs);
  return out;
}
inline std::string Deflate(const std::string &in) {
  z_stream zs{};
  if (deflateInit2(&zs, Z_DEFAULT_COMPRESSION, Z_DEFLATED, 16 + MAX_WBITS, 8, Z_DEFAULT_STRATEGY) != Z_OK)
    throw std::runtime_error("zlib deflateInit2 failed");
  zs.next_in = reinterpret_cast<Bytef *>(const_cast<char *>(in.data()));
  zs.avail_in = static_cast<uInt>(in.size());
  std::string out;
  char buf[1 << 16];
  int rc;
  do {
    zs.next_out = reinterpret_cast<Bytef *>(buf);
    zs.avail_out = sizeof(buf);
    rc = deflate(&zs, Z_FINISH);
    out.append(buf, sizeof(buf) - zs.avail_out);
  } while (rc == Z_OK);
  deflateEnd(&zs);
  return out;
}
}  // namespace shim

class filtering_istream : public std::istream {
 public:
  filtering_istream() : std::istream(&buf_) {}
  void push(const gzip_decompressor &) { gzip_ = true; }
  void push(std::istream &is) {
    std::string raw((std::istreambuf_iterator<char>(is)), std::istreambuf_iterator<char>());
    buf_.str(gzip_ ? shim::Inflate(raw) : raw);
  }
 private:
  std::stringbuf buf_;
  bool gzip_{false};
};

class filtering_ostream : public std::ostream {
 public:
  filtering_ostream() : std::ostream(&buf_) {}
  ~filtering_ostream() override {
    if (sink_ != nullptr) {
      const std::string data = buf_.str();
      const std::string out = gzip_ ? shim::Deflate(data) : data;
      sink_->write(out.data(), static_cast<std::streamsize>(out.size()));
      sink_->flush();
    }
  }
  void push(const gzip_compressor &) { gzip_ = true; }
  void push(std::ostream &os) { sink_ = &os; }
 private:
  std::stringbuf buf_;
  std::ostream *sink_{nullptr};
  bool gzip_{false};
};
}}  // namespace boost::iostreams
#endif
