/* sp_relax: the command line of sparse_relax.cpp:1165-1232 on the GPU
 * library (see nr_sp_relax_main). */
#include "netrelax.h"

int main(int argc, char **argv) { return nr_sp_relax_main(argc, argv); }
