// Storage for the single-rank MPI stand-in (test infrastructure only).
#include "mpi.h"

namespace MPI {
Intracomm COMM_WORLD;
}
