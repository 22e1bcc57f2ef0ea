/* Same single-rank MPI stand-in, for sources that include <mpi/mpi.h>. */
#pragma once
#include "../mpi.h"
