/* nmrelax: the command line of network_mesh_relax.cu:1424-1503 on the GPU
 * library (see nr_nmrelax_main). */
#include "netrelax.h"

int main(int argc, char **argv) { return nr_nmrelax_main(argc, argv); }
