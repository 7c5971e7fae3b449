/* Forced include for compiling the CPU regions of the reference's graphfdtd.cpp on their own:
 * the standard headers that file gets from its full include list, plus the two reference headers
 * the regions use (taken from the reference tree by -I). */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <iostream>
#include "Simple3DArray.h"
#include "graphfdtd.h"
using namespace std;
