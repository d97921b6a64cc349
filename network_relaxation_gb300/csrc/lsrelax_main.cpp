/* lsrelax: the command line of large_strain_relax.cu:1047-1126 on the GPU
 * library (see nr_lsrelax_main). */
#include "netrelax.h"

int main(int argc, char **argv) { return nr_lsrelax_main(argc, argv); }
