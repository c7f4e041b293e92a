// gzip filter tags for the filtering-stream stand-in. Test infrastructure only.
#ifndef LMC_ORACLE_SHIM_BOOST_IOSTREAMS_GZIP_
#define LMC_ORACLE_SHIM_BOOST_IOSTREAMS_GZIP_
namespace boost { namespace iostreams {
struct gzip_decompressor {};
struct gzip_compressor {};
}}  // namespace boost::iostreams
#endif
