/* Test stand-in: see ffstub.h. */
#include "ffstub.h"
