// ORACLE — TEST INFRASTRUCTURE ONLY.
// libguiding is an empty submodule in the reference; path.h includes this header but uses
// nothing from it beyond guiding/structures/btree.h.
#pragma once
#include "structures/btree.h"
