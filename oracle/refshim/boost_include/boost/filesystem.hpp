/* Stand-in for the part of Boost.Filesystem that na_calc.cpp uses (path,
 * directory_iterator, is_directory, exists): std::filesystem, whose
 * interface it mirrors.  Boost is not in this image; this header lets the
 * reference's own na_calc.cpp compile for the host so its non-affinity
 * (calc_na_val) can be called as a parity check. */
#ifndef NR_REF_BOOST_FILESYSTEM_HPP
#define NR_REF_BOOST_FILESYSTEM_HPP
#include <filesystem>
namespace boost {
namespace filesystem = std::filesystem;
}
#endif
