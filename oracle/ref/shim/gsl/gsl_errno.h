#pragma once
#include "../gsl_shim.h"
