// boost::filesystem::path(...).extension() is the only use in the reference's
// config I/O; std::filesystem provides the same member. Test infrastructure only.
#ifndef LMC_ORACLE_SHIM_BOOST_FILESYSTEM_
#define LMC_ORACLE_SHIM_BOOST_FILESYSTEM_
#include <filesystem>
namespace boost { namespace filesystem = std::filesystem; }
#endif
