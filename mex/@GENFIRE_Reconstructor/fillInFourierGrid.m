function obj = fillInFourierGrid(obj)
% Replaces @GENFIRE_Reconstructor/fillInFourierGrid.m (griddingMethod 1): FFT
% gridding on the GPU through genfire_mex.c and libgenfire.so (genfire_grid_fft).
[obj.measuredK, obj.recIFFT] = genfire_mex('grid_fft', obj);
end
