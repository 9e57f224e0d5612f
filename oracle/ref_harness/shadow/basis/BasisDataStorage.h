#pragma once
#include <basis/BasisManager.h>
