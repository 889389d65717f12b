// TEST INFRASTRUCTURE ONLY: the text-archive reader of this directory
// handles std::deque itself (boost/archive/text_iarchive.hpp).
#include <boost/serialization/access.hpp>
