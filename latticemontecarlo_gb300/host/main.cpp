// lmc_gb300 -p param.txt: the reference's command line (lmc/main.cpp, Home.cpp:97-125)
// for the KineticMcFirstOmp and CanonicalMcOmp methods, running on the GB300 kernels.
#include <exception>
#include <iostream>

#include "lmc_host.hpp"

int main(int argc, char *argv[]) {
  if (argc == 1) {
    std::cout << "No input parameter filename." << std::endl;
    return 1;
  }
  try {
    api::Parameter parameter(argc, argv);
    api::Run(parameter);
  } catch (const std::exception &e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
