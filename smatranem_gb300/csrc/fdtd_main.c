/* The drop-in `FDTD` command: `FDTD input.txt`, as SMatrAnEM's FDTD
 * (FDTDcalc/FDTDsplitfieldMetal.c main :32-187), running on the GPU. */
#include "smatran_fdtd.h"

int main(int argc, char **argv) { return smat_fdtd_main(argc, argv); }
