#pragma once
#include "phybs_qt_shim.h"
