/* Forwarding header of the hypre stand-in (see HYPRE.h). Test infrastructure. */
#include "HYPRE.h"
