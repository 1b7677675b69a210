// makeotf command-line program (the reference's src/otf/radialft.cpp main):
// `makeotf psf.tif otf.tif [switches]`.
#include <iostream>
#include <string>

#include "cudasirecon.h"

int main(int argc, char** argv)
{
  if (SRX_makeotfMain(argc, argv) != 0) {
    std::string e = SR_getLastError();
    if (e.rfind("usage:", 0) == 0) {
      std::cout << e << std::endl;
      return 0;
    }
    std::cerr << e << std::endl;
    return 1;
  }
  return 0;
}
