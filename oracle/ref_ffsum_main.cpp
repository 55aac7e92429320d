// Runs the reference's built-in delta-form-factor sum self-check
// (source/FormFactors.cpp:87-108, compiled with -D__SUM_TEST) for the hemicube
// side given on the command line and prints "ff sum: <value>" at 9 digits.
// TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <deque>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <list>
#include <sstream>
#include <string>
#include <vector>
#define private public
#include "Config.h"
#include "FormFactors.h"
#undef private
#include <cstdlib>
#include <iomanip>
#include <iostream>

int main(int argc, char** argv) {
    unsigned w = argc > 1 ? (unsigned)std::atoi(argv[1]) : 256;
    Config::setHemicubeSide(w);
    Config::setHemicubesCount(1);
    Config::freeze();
    std::cout << std::setprecision(9);
    float* t = precomputeHemicubeFormFactors();
    delete[] t;
    return 0;
}
