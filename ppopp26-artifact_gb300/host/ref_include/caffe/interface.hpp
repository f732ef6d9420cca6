// caffe/interface.hpp at the reference's include path (caffe/interface.hpp:1-29):
// a caller that includes "caffe/interface.hpp" and puts this directory on its
// include path gets this library's SyncedMemory instead of the reference's.
#pragma once
#include "../../syncedmem.h"
