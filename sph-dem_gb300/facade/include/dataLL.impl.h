/* Template definitions of CdataLL live in dataLL.h. */
#include "dataLL.h"
