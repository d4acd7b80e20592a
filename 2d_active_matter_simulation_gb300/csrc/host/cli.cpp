// `actflow` executable: the drop-in replacement of the reference program's
// command line (ActFlow_V3-2.cu:214-316).  All logic lives in libactflow.
#include "actflow.h"

int main(int argc, char **argv) { return am_cli_main(argc, argv); }
