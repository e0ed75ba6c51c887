/*
 * Test-infrastructure harness linked into the reference grid generator build
 * (oracle/build_ref.py: build_gridgen): the OpenMP thread count of its
 * parallel loops, and a way to run its main in a given working directory
 * (it writes a statistics text file under statistics/).
 */
#include <omp.h>
#include <unistd.h>

int ref_gridgen_main(int argc, char *argv[]);

void ref_set_num_threads(int n) { omp_set_num_threads(n); }
int ref_get_max_threads(void) { return omp_get_max_threads(); }

int ref_run_gridgen(const char *workdir, int argc, char *argv[])
{
    if (chdir(workdir) != 0) return -1;
    return ref_gridgen_main(argc, argv);
}
