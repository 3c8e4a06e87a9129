/* Stand-in for the one boost utility the reference uses: boost::next. */
#ifndef ORACLE_BOOST_UTILITY_SHIM
#define ORACLE_BOOST_UTILITY_SHIM
#include <iterator>
namespace boost {
template <class It> It next(It it, typename std::iterator_traits<It>::difference_type n = 1) {
    std::advance(it, n);
    return it;
}
}
#endif
