/* Stand-in for MPI when compiling the reference's one-rank files: only the
 * communicator type named in their signatures is needed. */
#pragma once
typedef int MPI_Comm;
