/* project-written stand-in: alphabet declarations live in the easel.h shim */
#include "easel.h"
