/* Stand-in for mpi.h -- TEST INFRASTRUCTURE ONLY.  The reference's CPU variant
 * includes it but calls no MPI routine ("wersja referencyjna/Wire_MoM.h":16). */
