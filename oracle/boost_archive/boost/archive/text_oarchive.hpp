// TEST INFRASTRUCTURE ONLY: the reference's GPU tool includes the writer
// but never writes an archive.
#ifndef GLS_ARCHIVE_STUB_OARCHIVE
#define GLS_ARCHIVE_STUB_OARCHIVE
#include <boost/serialization/access.hpp>
namespace boost { namespace archive { class text_oarchive {}; } }
#endif
