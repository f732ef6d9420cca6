// PLONK/utils/function.cuh at the reference's include path: the operator entry
// points (PLONK/utils/function.cuh:12-160), the quotient-constraint entry
// points of zkp/cuda/zksnark.cuh and the host field element
// cpu::BLS12_381_Fr_G1 (PLONK/utils/mont/cpu/ff/bls12-381.hpp:28-32), all
// from this library.  The standard headers are the ones the reference's header
// chain brings in and its drivers rely on (miss_ops.cu uses std::ifstream,
// std::chrono, std::thread and memcpy without including them itself).
#pragma once
#include <chrono>
#include <cstring>
#include <fstream>
#include <iostream>
#include <thread>

#include "../../../function.h"
#include "../../../zksnark.h"
