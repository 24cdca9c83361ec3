#pragma once
#include <thrust/device_vector.h>
