// TEST INFRASTRUCTURE
#pragma once
#include <memory>
