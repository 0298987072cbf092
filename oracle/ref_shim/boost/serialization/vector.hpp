// Oracle-only stub: std::vector serialization is never exercised by the oracle.
#pragma once
#include <vector>
