#pragma once
#include "trivial.hpp"
