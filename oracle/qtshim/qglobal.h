#pragma once
#include "qtshim.h"
