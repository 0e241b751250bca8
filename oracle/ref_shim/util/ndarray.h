// TEST INFRASTRUCTURE: empty stand-in (not used on the compiled path)
#pragma once
#include "util/stats.h"
