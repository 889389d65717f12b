// Empty stub (TEST INFRASTRUCTURE ONLY).
#include "access.hpp"
