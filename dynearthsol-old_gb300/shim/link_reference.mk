# Links the reference program -- dynearthsol.cxx and the rest of its sources,
# unchanged -- with its hot-path functions taken from the GPU library: the
# shim (des_shim_functions.cpp) defines update_temperature, update_strain_rate,
# compute_dvoldt, compute_edvoldt, update_stress, NMD_stress, update_force,
# update_velocity, apply_vbcs, update_coordinate, compute_volume,
# compute_mass, compute_shape_fn, rotate_stress and compute_dt with the
# reference's own signatures; the reference's definitions of exactly those
# symbols are made weak in copies of its objects (objcopy --weaken-symbol), so
# every call to them -- from the loop body, init, restart, remesh -- binds to
# the shim at link time.  Nothing in the reference's sources changes.
#
#   make -f dynearthsol-old_gb300/shim/link_reference.mk REF=<reference tree> \
#        OUT=<build dir> [INPUT_OBJ=<object defining get_input_parameters>] -j8
#
# INPUT_OBJ defaults to the reference's input.cxx (it needs boost's
# program_options, -lboost_program_options); a build without boost passes an
# object of its own.  Flags are the reference's Makefile defaults (opt=2
# openmp=1 ndims=3); NVTX (included by dynearthsol.cxx) comes from CUDA.
REF    ?=
OUT    ?= dynearthsol-old_gb300/_build/ref_link
ROOT   := $(patsubst %/dynearthsol-old_gb300/shim/,%,$(dir $(abspath $(lastword $(MAKEFILE_LIST)))))
SHIM   := $(ROOT)/dynearthsol-old_gb300/shim
LIBDIR := $(ROOT)/dynearthsol-old_gb300/_build
CUDA   ?= /usr/local/cuda
CXX    ?= g++
BASE   := -std=c++0x -fPIC -fopenmp -DTHREED -I$(REF) -I$(REF)/ann/include -I$(CUDA)/include/nvtx3 -w
CXXFLAGS := $(BASE) -O2
OBJ    := $(OUT)/obj
WEAK   := $(OUT)/weak

ifeq ($(REF),)
$(error REF=<reference tree> is required)
endif

DES_SRCS := dynearthsol fields geometry rheology matprops bc mesh markerset barycentric-fn binaryio \
            output ic ic-read-temp brc-interpolation phasechanges remeshing nn-interpolation
C3X3     := dsytrd3 dsyevc3 dsyevq3 dsyevh3
ANN_SRCS := ANN brute kd_tree kd_util kd_split kd_dump kd_search kd_pr_search \
            kd_fix_rad_search bd_tree bd_search bd_pr_search bd_fix_rad_search perf

REF_OBJS := $(addprefix $(OBJ)/,$(addsuffix .o,$(DES_SRCS))) \
            $(addprefix $(OBJ)/3x3_,$(addsuffix .o,$(C3X3))) \
            $(addprefix $(OBJ)/ann_,$(addsuffix .o,$(ANN_SRCS))) \
            $(OBJ)/predicates.o $(OBJ)/tetgen.o $(OBJ)/triangle.o
WEAK_OBJS := $(patsubst $(OBJ)/%,$(WEAK)/%,$(REF_OBJS))
SHIM_OBJS := $(OUT)/des_shim.o $(OUT)/des_shim_functions.o

ifeq ($(INPUT_OBJ),)
INPUT_OBJ := $(OBJ)/input.o
INPUT_LIB := -lboost_program_options
endif

all: $(OUT)/dynearthsol3d_gpu

$(OBJ) $(WEAK):
	mkdir -p $@

$(OBJ)/%.o: $(REF)/%.cxx | $(OBJ)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OBJ)/3x3_%.o: $(REF)/3x3-C/%.c | $(OBJ)
	$(CXX) -fPIC -O3 -ffast-math -w -c $< -o $@

$(OBJ)/ann_%.o: $(REF)/ann/src/%.cpp | $(OBJ)
	$(CXX) -fPIC -O2 -w -I$(REF)/ann/include -c $< -o $@

$(OBJ)/predicates.o: $(REF)/tetgen/predicates.cxx | $(OBJ)
	$(CXX) $(BASE) -DTETLIBRARY -O0 -c $< -o $@

$(OBJ)/tetgen.o: $(REF)/tetgen/tetgen.cxx | $(OBJ)
	$(CXX) $(BASE) -O2 -DNDEBUG -DTETLIBRARY -c $< -o $@

$(OBJ)/triangle.o: $(REF)/triangle/triangle.c | $(OBJ)
	$(CXX) $(BASE) -O1 -DTRILIBRARY -DREDUCED -DANSI_DECLARATORS -c $< -o $@

$(OUT)/%.o: $(SHIM)/%.cpp $(SHIM)/des_shim_internal.hpp $(ROOT)/include/des_gpu.h
	$(CXX) $(CXXFLAGS) -I$(ROOT)/include -I$(SHIM) -c $< -o $@

# the global functions the shim defines, mangled
$(OUT)/shim_symbols.txt: $(OUT)/des_shim_functions.o
	nm -g --defined-only $< | awk '$$2 == "T" {print $$3}' > $@

$(WEAK)/%.o: $(OBJ)/%.o $(OUT)/shim_symbols.txt | $(WEAK)
	objcopy $$(sed 's/^/--weaken-symbol=/' $(OUT)/shim_symbols.txt) $< $@

$(OUT)/dynearthsol3d_gpu: $(WEAK_OBJS) $(SHIM_OBJS) $(INPUT_OBJ) $(LIBDIR)/libdes_gb300.so
	$(CXX) -fopenmp -o $@ $(WEAK_OBJS) $(SHIM_OBJS) $(INPUT_OBJ) -L$(LIBDIR) -ldes_gb300 \
	    -Wl,-rpath,$(LIBDIR) $(INPUT_LIB) $(LINK_EXTRA)

.PHONY: all
# keep the reference objects between runs (make would delete them as intermediates)
.SECONDARY:
