#pragma once
#include "operator.h"
