/* Case-fix for the reference's #include "partition.h" (the file is Partition.h). */
#pragma once
#include "Partition.h"
