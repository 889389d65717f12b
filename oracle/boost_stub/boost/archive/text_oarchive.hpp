// Empty stub (TEST INFRASTRUCTURE ONLY).
#include "../serialization/access.hpp"
