// TEST INFRASTRUCTURE: see fmt/format.h
#pragma once
#include "fmt/format.h"
