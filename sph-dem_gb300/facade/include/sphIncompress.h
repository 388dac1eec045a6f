/*
 * The step class of the reference (sphIncompress.h CsphIncompress).  The
 * device runs the step, so case code sees the class by name only: output
 * code such as customOutput's calcPostProcess takes a pointer to it.  The
 * header also brings in what the reference's sphIncompress.h brings in for
 * case code: the data structure and the Nsph helpers.
 */
#ifndef SPHINCOMPRESS_H
#define SPHINCOMPRESS_H

#include "dataLL.h"
#include "sph.h"

class CsphIncompress;

#endif
