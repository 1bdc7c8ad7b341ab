// The reference includes LinearMapping.h under this spelling; the file system here is case-sensitive.
#pragma once
#include "LinearMapping.h"
