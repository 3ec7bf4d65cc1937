# Test infrastructure: builds the UNMODIFIED reference (spaceauk/AMR2D_MHD)
# from its sources where they lie, plus oracle/ref_hook.cpp, into oracle/_ref/.
# Nothing is copied: the generated sources are defs.hpp with `maxlevs`
# replaced (it is a compile-time constant in the reference, defs.hpp:28), and
# `-I-` makes the compiler pick that header instead of the one beside the
# sources (likewise `nghosts`, defs.hpp:27, which WENO5 needs at 4); with
# ROTOR_G53=1 also IC2Dtype.cpp with the rotor's gamma (IC2Dtype.cpp:77,
# 1.4) replaced by 5.0/3.0.  main.cpp is compiled with two renames (see
# ref_hook.cpp).
#
# REF (the reference checkout) has no default: pass it, or export
# AMR_REFERENCE_SRC.
#
#   make -f oracle/ref.mk REF=<src> MAXLEVS=4 FLAVOR=shipped   # makefile:9-13 flags
#   make -f oracle/ref.mk REF=<src> MAXLEVS=4 FLAVOR=nofma     # same + -ffp-contract=off
#   make -f oracle/ref.mk REF=<src> MAXLEVS=4 FLAVOR=omp       # same as shipped + USE_OMP
#   make -f oracle/ref.mk REF=<src> MAXLEVS=4 FLAVOR=nofma CTTYPE=2 DIFFUSION=true
#   make -f oracle/ref.mk REF=<src> MAXLEVS=5 FLAVOR=nofma ROTOR_G53=1
#   make -f oracle/ref.mk REF=<src> FLAVOR=nofma MAGFIELD=false kat
#
# The result is oracle/_ref/L<MAXLEVS>_G<NGHOSTS>_<FLAVOR>[_CT2][_DIFF][_RG53][_HYDRO]/main.x;
# run it in a directory holding input.txt with stdin "2\n0\n" (main.cpp:75,275).
# The omp flavour is for timing only: its dt loop (main.cpp:215-223) updates
# the shared lambda1 / lambda2 from every thread without a reduction.

REF     ?= $(AMR_REFERENCE_SRC)
ifeq ($(strip $(REF)),)
$(error REF is not set: pass REF=<reference checkout> or export AMR_REFERENCE_SRC)
endif
MAXLEVS ?= 5
NGHOSTS ?= 2
FLAVOR  ?= shipped
# CTtype (defs.hpp:34, 1 basic / 2 upwind) and diffusion (defs.hpp:35), also
# compile-time constants of the reference; non-default values get their own
# build directory
CTTYPE    ?= 1
DIFFUSION ?= false
# 1: the rotor IC with gamma = 5/3 instead of the reference's 1.4
ROTOR_G53 ?= 0
# MAG_field (defs.hpp:32): false builds the reference's hydrodynamic
# configuration, the only one in which riemannS reaches ROE (riemannS.cpp:39)
MAGFIELD ?= true
HERE    := $(dir $(lastword $(MAKEFILE_LIST)))
VARIANT := $(if $(filter-out 1,$(CTTYPE)),_CT$(CTTYPE))$(if $(filter true,$(DIFFUSION)),_DIFF)$(if $(filter 1,$(ROTOR_G53)),_RG53)$(if $(filter false,$(MAGFIELD)),_HYDRO)
OUT     := $(HERE)_ref/L$(MAXLEVS)_G$(NGHOSTS)_$(FLAVOR)$(VARIANT)

CXX     ?= g++
# makefile:9-13 of the reference
CFLAGS  := -O3 -std=c++17 -march=native -funroll-loops -g -DDOUBLE_PREC -w
LFLAGS  :=
ifeq ($(FLAVOR),nofma)
CFLAGS  += -ffp-contract=off
endif
ifeq ($(FLAVOR),omp)
CFLAGS  += -fopenmp -DOPENMP
LFLAGS  += -fopenmp
endif

# every reference translation unit except savedata.cpp (text output, replaced
# by the hook's no-op) and main.cpp (built with renames below)
SRCS := meshblock IC2Dtype MUSCL2D slopelimiter celledges riemannS \
        WENO2D_primvar parameters diffusivity timeIntegral basegrid \
        locate_bounds boundary extboundary markref criteria critneighup \
        critneighdown refine coarsen updatelpup updatelpdown admesh misc \
        CT2D refineBi_CT coarsenBi_CT boundaryfc boundaryec
OBJS := $(addprefix $(OUT)/,$(addsuffix .o,$(SRCS))) $(OUT)/main.o $(OUT)/ref_hook.o
INC  := -I- -I$(OUT) -I$(REF)

all: $(OUT)/main.x

# known-answer harness on the reference's own riemannS / misc / slopelimiter
kat: $(OUT)/kat.x

$(OUT)/ref_kat.o: $(HERE)ref_kat.cpp $(OUT)/defs.hpp
	$(CXX) -c $(CFLAGS) $(INC) $< -o $@

$(OUT)/kat.x: $(OUT)/ref_kat.o $(OUT)/riemannS.o $(OUT)/misc.o $(OUT)/slopelimiter.o
	$(CXX) $(LFLAGS) $^ -o $@

$(OUT)/defs.hpp: $(REF)/defs.hpp
	@mkdir -p $(OUT)
	sed -e 's/^const int maxlevs=5;/const int maxlevs=$(MAXLEVS);/' \
	    -e 's/^const int nghosts=2; /const int nghosts=$(NGHOSTS); /' \
	    -e 's/^const int CTtype=1;/const int CTtype=$(CTTYPE);/' \
	    -e 's/^const bool diffusion=false;/const bool diffusion=$(DIFFUSION);/' \
	    -e 's/^const bool MAG_field=true;/const bool MAG_field=$(MAGFIELD);/' $< > $@
	@grep -q 'const int maxlevs=$(MAXLEVS);' $@ || (echo "maxlevs patch failed" && rm -f $@ && false)
	@grep -q 'const int nghosts=$(NGHOSTS); ' $@ || (echo "nghosts patch failed" && rm -f $@ && false)
	@grep -q 'const int CTtype=$(CTTYPE);' $@ || (echo "CTtype patch failed" && rm -f $@ && false)
	@grep -q 'const bool diffusion=$(DIFFUSION);' $@ || (echo "diffusion patch failed" && rm -f $@ && false)
	@grep -q 'const bool MAG_field=$(MAGFIELD);' $@ || (echo "MAG_field patch failed" && rm -f $@ && false)

# the rotor branch of IC2Dtype.cpp (between IC=="rotor" and its tEnd) with
# gamma = 5/3; exactly one line changes
$(OUT)/IC2Dtype_g53.cpp: $(REF)/IC2Dtype.cpp
	@mkdir -p $(OUT)
	sed -e '/IC=="rotor"/,/tEnd=0.295/ s/gamma=1\.4;/gamma=5.0\/3.0;/' $< > $@
	@test "$$(diff $< $@ | grep -c '^>')" = 1 || (echo "rotor gamma patch failed" && rm -f $@ && false)
	@grep -q 'gamma=5.0/3.0;' $@ || (echo "rotor gamma patch failed" && rm -f $@ && false)

ifeq ($(ROTOR_G53),1)
$(OUT)/IC2Dtype.o: $(OUT)/IC2Dtype_g53.cpp $(OUT)/defs.hpp
	$(CXX) -c $(CFLAGS) $(INC) $< -o $@
endif

$(OUT)/%.o: $(REF)/%.cpp $(OUT)/defs.hpp
	$(CXX) -c $(CFLAGS) $(INC) $< -o $@

$(OUT)/main.o: $(REF)/main.cpp $(OUT)/defs.hpp
	$(CXX) -c $(CFLAGS) $(INC) -Dadmesh=amr_ref_admesh_hook -Dsave4py=amr_ref_save4py $< -o $@

$(OUT)/ref_hook.o: $(HERE)ref_hook.cpp $(OUT)/defs.hpp
	$(CXX) -c $(CFLAGS) $(INC) $< -o $@

$(OUT)/main.x: $(OBJS)
	$(CXX) $(LFLAGS) $(OBJS) -o $@

.PHONY: all kat
