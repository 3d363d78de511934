// Stand-in for Eigen's test harness header when Eigen's own test files are compiled against the
// GB300 backend (tests/test_eigen_backend.py): the harness must come before any Eigen header (it
// redefines eigen_assert), and the backend header must come before the test body instantiates
// LLT.  Compiled with `-I <this dir> -I-` so that the tests' #include "main.h" lands here.
#include EIGEN_TEST_HARNESS
#include "eigen_gb300/LLT_GB300.h"
