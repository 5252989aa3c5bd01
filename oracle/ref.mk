# Builds oracle/_ref/libsfref.so: the reference's own hot-path sources, compiled where they lie (REF) against
# the stand-in headers in oracle/refshim, plus oracle/ref_driver.cpp.  TEST INFRASTRUCTURE: it pins the
# oracle; nothing in the library links it.  The reference's own build system (xmake) is not used.
#
#   make -f oracle/ref.mk REF=/root/reference
REF ?= /root/reference
HERE := $(dir $(lastword $(MAKEFILE_LIST)))
OUT := $(HERE)_ref
CXX ?= g++
CXXFLAGS := -std=c++20 -O2 -fPIC -ffp-contract=off -w -I$(HERE)refshim -I$(REF)/core
SRCS := $(REF)/core/Pressure.cpp $(REF)/core/MagneticField.cpp $(REF)/core/Collider.cpp \
        $(REF)/core/FastMarching.cpp $(REF)/core/Extrapolation.cpp $(REF)/core/Reinitialization.cpp $(REF)/core/CSG.cpp \
        $(HERE)ref_driver.cpp
OBJS := $(patsubst %.cpp,$(OUT)/%.o,$(notdir $(SRCS)))
SHIM := $(wildcard $(HERE)refshim/*/* $(HERE)refshim/*/*/*)

$(OUT)/libsfref.so: $(OBJS)
	$(CXX) -shared -o $@ $(OBJS)

$(OUT)/%.o: $(REF)/core/%.cpp $(SHIM) | $(OUT)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT)/ref_driver.o: $(HERE)ref_driver.cpp $(SHIM) | $(OUT)
	$(CXX) $(CXXFLAGS) -c $< -o $@

$(OUT):
	mkdir -p $@

.PHONY: clean
clean:
	rm -f $(OUT)/*.o $(OUT)/libsfref.so
