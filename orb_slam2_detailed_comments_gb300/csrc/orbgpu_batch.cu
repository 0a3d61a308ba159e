#include "orbgpu_host.h"
