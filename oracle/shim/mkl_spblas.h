#pragma once
#include "mkl.h"
