/* Namespace of the case-side helpers (misc.h Nmisc); hook code only needs
 * the namespace and the math headers. */
#ifndef SPHDEM_FACADE_MISC_H
#define SPHDEM_FACADE_MISC_H

#include <cmath>
#include <iostream>

#include "particle.h"

using namespace std;

namespace Nmisc {}

#endif
