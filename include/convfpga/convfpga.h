/* Forwarding header: programs written against pc2/ConvFPGA include
 * "convfpga/convfpga.h" (src/main.cpp:5-7); the declarations live in ../convfpga.h. */
#include "../convfpga.h"
