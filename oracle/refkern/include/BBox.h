// The reference's primitive.h includes "BBox.h" while the file on disk is
// bbox.h (it was written on a case-insensitive file system); forward to it.
#pragma once
#include <bbox.h>
