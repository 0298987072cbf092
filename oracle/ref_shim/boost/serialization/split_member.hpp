// Oracle-only stub for BOOST_SERIALIZATION_SPLIT_MEMBER (no archive is ever used).
#pragma once
#include "access.hpp"
#define BOOST_SERIALIZATION_SPLIT_MEMBER()
