# TEST INFRASTRUCTURE -- builds the reference's own hot-path sources, where
# they lie, into oracle/_ref/libdesref.so together with oracle/ref_harness.cpp.
# The reference's build system is not used; the flags are its defaults
# (Makefile: opt=2 openmp=1 ndims=3 -> -O2 -fopenmp -DTHREED; 3x3-C with
# -O3 -ffast-math as 3x3-C/Makefile sets; TetGen predicates at -O0; Triangle at
# -O1).  input.cxx (boost) and dynearthsol.cxx (main) are not built.
#
#   make -f oracle/ref.mk REF=<reference tree> -j8     (oracle.build_ref() passes it)
REF    ?=
ifeq ($(REF),)
$(error REF=<reference tree> is required)
endif
OUT    := oracle/_ref
OBJ    := $(OUT)/obj
CXX    ?= g++
BASE   := -std=c++0x -fPIC -fopenmp -DTHREED -I$(REF) -I$(REF)/ann/include -w
CXXFLAGS := $(BASE) -O2

DES_SRCS := fields geometry rheology matprops bc mesh markerset barycentric-fn binaryio output \
            ic ic-read-temp brc-interpolation phasechanges
C3X3     := dsytrd3 dsyevc3 dsyevq3 dsyevh3
ANN_SRCS := ANN brute kd_tree kd_util kd_split kd_dump kd_search kd_pr_search \
            kd_fix_rad_search bd_tree bd_search bd_pr_search bd_fix_rad_search perf

OBJS := $(addprefix $(OBJ)/,$(addsuffix .o,$(DES_SRCS))) \
        $(addprefix $(OBJ)/3x3_,$(addsuffix .o,$(C3X3))) \
        $(addprefix $(OBJ)/ann_,$(addsuffix .o,$(ANN_SRCS))) \
        $(OBJ)/predicates.o $(OBJ)/tetgen.o $(OBJ)/triangle.o

all: $(OUT)/libdesref.so

$(OBJ):
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

$(OBJ)/ref_harness.o: oracle/ref_harness.cpp | $(OBJ)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/libdesref.so: $(OBJS) $(OBJ)/ref_harness.o
	$(CXX) -shared -fopenmp -o $@ $^ -lm

.PHONY: all
