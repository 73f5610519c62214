#include "mlvalues.h"
