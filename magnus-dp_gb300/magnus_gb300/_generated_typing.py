from typing import Literal

NumericBackendName = Literal["float", "double", "std::complex<float>", "std::complex<double>"]
MatrixBackendName = Literal["Fixed2", "Manual", "Blas", "SpaceCurve", "GB300", "Auto"]
IntegratorName = Literal["Boole", "Simpson", "Trapezoid", "Riemann", "Auto"]
GLBackendName = Literal["threadpool", "openmp", "serial", "Auto"]
KernelOpName = Literal["one", "many", "sum"]
PrecisionName = Literal["plain", "mixed"]
