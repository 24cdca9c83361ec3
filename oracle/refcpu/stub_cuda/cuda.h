/* Empty stand-in for the CUDA driver header when the reference's device
 * code is compiled as host C++ for the CPU oracle (test infrastructure). */
#pragma once
