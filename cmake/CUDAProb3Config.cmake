# CMake package for the GB300 propagator library, with the target names CUDAProb3++ exports
# (CUDAProb3::CUDAProb3Atmos, CUDAProb3::CUDAProb3Beam), so a project that links them gets
# libcp3gb300.so and the compatible headers instead:
#
#   find_package(CUDAProb3 CONFIG REQUIRED PATHS <repo>/cmake)
#   target_link_libraries(app PRIVATE CUDAProb3::CUDAProb3Atmos)
#
# Build the library first: python -m cudaprob3_gb300.build
get_filename_component(_cp3_root "${CMAKE_CURRENT_LIST_DIR}/.." ABSOLUTE)
set(_cp3_lib "${_cp3_root}/cudaprob3_gb300/_lib/libcp3gb300.so")
if(NOT EXISTS "${_cp3_lib}")
  set(CUDAProb3_FOUND FALSE)
  set(CUDAProb3_NOT_FOUND_MESSAGE "libcp3gb300.so not built: run `python -m cudaprob3_gb300.build` in ${_cp3_root}")
  return()
endif()
if(NOT TARGET CUDAProb3::cp3gb300)
  add_library(CUDAProb3::cp3gb300 SHARED IMPORTED)
  set_target_properties(CUDAProb3::cp3gb300 PROPERTIES
    IMPORTED_LOCATION "${_cp3_lib}"
    INTERFACE_INCLUDE_DIRECTORIES "${_cp3_root}/include;${_cp3_root}/include/compat"
    INTERFACE_COMPILE_FEATURES cxx_std_14)
  add_library(CUDAProb3::CUDAProb3Atmos INTERFACE IMPORTED)
  set_target_properties(CUDAProb3::CUDAProb3Atmos PROPERTIES INTERFACE_LINK_LIBRARIES CUDAProb3::cp3gb300)
  add_library(CUDAProb3::CUDAProb3Beam INTERFACE IMPORTED)
  set_target_properties(CUDAProb3::CUDAProb3Beam PROPERTIES INTERFACE_LINK_LIBRARIES CUDAProb3::cp3gb300)
endif()
set(CUDAProb3_FOUND TRUE)
