/* Case-fix for the reference's #include "Writer.h" (the file is writer.h). */
#pragma once
#include "writer.h"
