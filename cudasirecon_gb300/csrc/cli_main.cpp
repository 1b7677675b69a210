// cudasirecon command-line driver (src/cudaSirecon/cudaSireconDriver.cpp:5-27):
// construct from argv, then per time point setFile -> loadAndRescaleImage ->
// setCurTimeIdx -> processOneVolume -> writeResult, then closeFiles.
#include <cstdio>
#include <cstring>
#include <iostream>
#include <string>

#include "cudasirecon.h"

int main(int argc, char** argv)
{
  SIM_Reconstructor* r = SR_new_from_argv(argc, argv);
  if (!r) {
    std::string e = SR_getLastError();
    if (e.rfind("help requested", 0) == 0) {
      std::cout << "cudasirecon (GB300 build)\n\n" << e.substr(strlen("help requested\n")) << std::endl;
      return 0;
    }
    if (e == "version requested") {
      std::cout << "Version 1.2.0-gb300" << std::endl;
      return 0;
    }
    // the reference reports and still exits with status 0 (cudaSireconDriver.cpp:22-25)
    std::cerr << "\n!!Error occurred: " << e << std::endl;
    return 0;
  }
  int nt = SR_getNTimes(r);
  for (int it = 0; it < nt; ++it) {
    for (int iw = 0; iw < 1; ++iw) {
      SR_clearError();
      SR_setFile(r, it, iw);
      SR_loadAndRescaleImage(r, it, iw);
      SR_setCurTimeIdx(r, it);
      SR_processOneVolume(r);
      if (SRX_lastProcessResult(r) == 1) SR_writeResult(r, it, iw);
      if (*SR_getLastError()) {
        std::cerr << "\n!!Error occurred: " << SR_getLastError() << std::endl;
        SR_delete(r);
        return 0;
      }
      std::printf("Time point %d, wave %d done\n", it, iw);
    }
  }
  SR_closeFiles(r);
  SR_delete(r);
  return 0;
}
