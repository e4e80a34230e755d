// util/PlatformUtils.hpp — forwards to the DOM subset in shim_dom.hpp (test infrastructure).
#include "../shim_dom.hpp"
