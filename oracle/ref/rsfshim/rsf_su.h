#include "rsf.h"
