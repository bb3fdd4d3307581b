{-# LANGUAGE CPP                 #-}
{-# LANGUAGE FlexibleContexts    #-}
{-# LANGUAGE ScopedTypeVariables #-}
{-# LANGUAGE TypeOperators       #-}
-- |
-- Module      : Data.Array.Accelerate.Math.FFT.SpecConv
--
-- Spectral convolution of a batch of 3D fields with one filter spectrum,
--
--   y_b = fft3D Inverse (fft3D Forward x_b * H),
--
-- and its vector-Jacobian product for L(y): given g_y = dL/dy it returns
--
--   g_Y = Forward(g_y) / N,   g_H = sum_b conj(X_b) * g_Y_b,
--   g_x = Reverse(conj H * g_Y),   X_b = Forward(x_b) recomputed,
--
-- with N = d*h*w, in the conjugate-Wirtinger convention (for L = 1/2 |y|^2,
-- g_y = y).  On the PTX backend both run as libgbfft's fused kernels
-- (LLVM.PTX.SpecConv); elsewhere the same formulas are composed from the
-- innermost-axis `fft` and axis rotations, as the reference composes fft3D
-- (FFT.hs:150-187).  Written against accelerate 1.3 and not compiled here
-- (no GHC in this environment).
--
module Data.Array.Accelerate.Math.FFT.SpecConv (

  specConv,
  specConvVJP,

) where

import Data.Array.Accelerate                                        as A
import Data.Array.Accelerate.Data.Complex
import Data.Array.Accelerate.Math.FFT                               ( Mode(..), fft )
#ifdef ACCELERATE_LLVM_PTX_BACKEND
import qualified Data.Array.Accelerate.Math.FFT.LLVM.PTX.SpecConv   as PTX
#endif

type Fields = Array DIM4 (Complex Float)
type Spectrum = Array DIM3 (Complex Float)

-- | y = Inverse3D (Forward3D x * H) for every field x_b of the batch.
specConv :: Acc Fields -> Acc Spectrum -> Acc Fields
specConv x h =
  go (T2 x h)
  where
    go =
#ifdef ACCELERATE_LLVM_PTX_BACKEND
      foreignAcc PTX.specConv $
#endif
      \(T2 x' h') -> spectral3 Inverse (A.zipWith (*) (spectral3 Forward x') (overBatch x' h'))

-- | (g_x, g_H) for the cotangent g_y of y = specConv x h.
specConvVJP :: Acc Fields -> Acc Spectrum -> Acc Fields -> Acc (Fields, Spectrum)
specConvVJP x h gy =
  go (T3 x h gy)
  where
    go =
#ifdef ACCELERATE_LLVM_PTX_BACKEND
      foreignAcc PTX.specConvVJP $
#endif
      \(T3 x' h' gy') ->
        let Z :. _ :. d :. hh :. w = unlift (shape x') :: Z :. Exp Int :. Exp Int :. Exp Int :. Exp Int
            n   = A.fromIntegral (d * hh * w) :: Exp (Complex Float)
            gY  = A.map (/ n) (spectral3 Forward gy')
            xX  = spectral3 Forward x'
            gx  = spectral3 Reverse (A.zipWith (*) (A.map conjugate (overBatch x' h')) gY)
            gh  = sumBatch (A.zipWith (*) (A.map conjugate xX) gY)
        in  T2 gx gh

-- The 3D transform of every field: the innermost-axis transform three times,
-- rotating the three inner axes after each (Inverse divides by each extent).
spectral3 :: Mode -> Acc Fields -> Acc Fields
spectral3 mode = rot . fft mode >-> rot . fft mode >-> rot . fft mode
  where
    rot a = let Z :. b :. z :. y :. x = unlift (shape a) :: Z :. Exp Int :. Exp Int :. Exp Int :. Exp Int
            in  backpermute (lift (Z :. b :. y :. x :. z))
                            (\ix -> let Z :. b' :. y' :. x' :. z' = unlift ix :: Z :. Exp Int :. Exp Int :. Exp Int :. Exp Int
                                    in  lift (Z :. b' :. z' :. y' :. x'))
                            a

-- H repeated along the batch axis of x.
overBatch :: Acc Fields -> Acc Spectrum -> Acc Fields
overBatch x h =
  let Z :. b :. _ :. _ :. _ = unlift (shape x) :: Z :. Exp Int :. Exp Int :. Exp Int :. Exp Int
  in  A.replicate (lift (Z :. b :. All :. All :. All)) h

-- Sum over the batch (outermost) axis.
sumBatch :: Acc Fields -> Acc Spectrum
sumBatch a =
  A.sum (backpermute (let Z :. b :. z :. y :. x = unlift (shape a) :: Z :. Exp Int :. Exp Int :. Exp Int :. Exp Int
                      in  lift (Z :. z :. y :. x :. b))
                     (\ix -> let Z :. z :. y :. x :. b = unlift ix :: Z :. Exp Int :. Exp Int :. Exp Int :. Exp Int
                             in  lift (Z :. b :. z :. y :. x))
                     a)
