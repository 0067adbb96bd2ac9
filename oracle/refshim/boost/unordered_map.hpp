#pragma once
#include "shim_all.hpp"
