# Builds the reference's FastChem (fastchem_vulcan, C++, the engine behind
# ini_mix = 'EQ', build_atm.py:78-164) from its sources where they lie into
# oracle/_ref/fastchem.  Test infrastructure only: the equilibrium fixture
# (tests/golden/make_fastchem_golden.py) runs it; nothing else does.
#   make -f oracle/fastchem.mk REF=<path of the VULCAN tree>
ifndef REF
$(error give the VULCAN source tree: make -f oracle/fastchem.mk REF=<path>)
endif
FC   = $(REF)/fastchem_vulcan
SRC  = $(wildcard $(FC)/fastchem_src/*.cpp) $(FC)/model_main/model_main.cpp \
       $(FC)/model_main/read_config.cpp
OUT  = $(dir $(lastword $(MAKEFILE_LIST)))_ref/fastchem

$(OUT): $(SRC)
	mkdir -p $(dir $@)
	g++ -O2 -std=gnu++11 -w $(SRC) -o $@ -lm
