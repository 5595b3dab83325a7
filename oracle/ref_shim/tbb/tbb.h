// Stand-in for <tbb/tbb.h> (see tbb/mutex.h).
#pragma once
#include "tbb/mutex.h"
