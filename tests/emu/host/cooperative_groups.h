// Test infrastructure: the cluster subset of cooperative groups (see ../fake).
#pragma once
#include "../fake/cooperative_groups.h"
