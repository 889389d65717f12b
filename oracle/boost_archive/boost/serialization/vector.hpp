// TEST INFRASTRUCTURE ONLY: the text-archive reader of this directory
// handles std::vector itself (boost/archive/text_iarchive.hpp).
#include <boost/serialization/access.hpp>
