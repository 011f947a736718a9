#pragma once
#include "detail/_range_common.h"
