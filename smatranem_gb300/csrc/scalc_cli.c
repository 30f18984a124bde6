/* The drop-in `Scalc` command: `Scalc input.txt`, as SMatrAnEM's S-matrix
 * program (Smat/Scalc.c main :27-96), with the layer transfer on the GPU. */
#include "smatran_fdtd.h"

int main(int argc, char **argv) { return smat_scalc_main(argc, argv); }
