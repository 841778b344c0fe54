// declaration-only stand-in (see refstubs_decls.hpp)
#include "refstubs_decls.hpp"
