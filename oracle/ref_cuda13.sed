# Edits that let the reference program (cuDebye-v15.cu, written for MSVC and
# CUDA 8) compile with nvcc 13 and gcc 13 on Linux. Applied by `make ref` to a
# copy under oracle/_ref/; the arithmetic of the kernels is not touched.
#  - thrust::identity is gone from CUDA 13's Thrust: use cuda::std::identity
#    as the copy_if predicate (a non-zero count is true), :326
s|#include <thrust/copy.h>|#include <thrust/copy.h>\n#include <cuda/std/functional>|
s|thrust::identity<unsigned int>()|cuda::std::identity()|
#  - MSVC-only functional casts to a multi-word type, :344, :365-366, :544-547
s|long long unsigned int(\([^()]*\))|(unsigned long long)(\1)|g
#  - main must return int, :599; its early exits, :621, :832, :1003
s|^void main(int argc, char\* argv\[\])|int main(int argc, char* argv[])|
599,$s|^\t\treturn;|\t\treturn 1;|
599,$s|^\treturn;|\treturn 0;|
#  - cudaDeviceProp lost clockRate and kernelExecTimeoutEnabled in CUDA 13
#    (two information prints), :661-662
/prop\.clockRate/d
/prop\.kernelExecTimeoutEnabled/d
