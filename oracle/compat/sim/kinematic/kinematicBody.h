// The reference's collision sources include this header with a lower-case
// "k" (its Windows build does not mind the case); the file is KinematicBody.h.
#pragma once
#include "sim/kinematic/KinematicBody.h"
