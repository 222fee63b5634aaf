// Stand-in header of the external beadrodpmer library (test infrastructure).
#pragma once
#include "beadrodpmer/chain_standin.hpp"
