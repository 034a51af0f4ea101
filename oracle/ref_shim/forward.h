// Declaration-only stand-in (see forward_vector.h). Test infrastructure only.
#pragma once
#include "forward_vector.h"
