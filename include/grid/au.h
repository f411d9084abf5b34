/* libdft drivers include <grid/au.h>; with -I<repo>/include this header gives
 * them the libdftgpu declarations (the same names and signatures). */
#include "../dftgpu.h"
