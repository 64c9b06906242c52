// see ../random.hpp
#pragma once
#include "boost/random.hpp"
