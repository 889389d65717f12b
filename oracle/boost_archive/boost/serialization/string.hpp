// TEST INFRASTRUCTURE ONLY: the text-archive reader of this directory
// handles std::string itself (boost/archive/text_iarchive.hpp).
#include <boost/serialization/access.hpp>
