// Compat stand-in (test infrastructure).
#pragma once
#include "glog/logging.h"
