#pragma once
#include "../tbb/tbb.h"
